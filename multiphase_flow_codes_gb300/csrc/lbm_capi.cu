// lbm_capi.cu - the C ABI (include/lbm.h) over the GB300 kernels.
//
// A context owns every device buffer of one box.  Populations are kept in
// the "plain" post-streaming layout between calls, which is the state the
// reference holds between its subroutines, so the per-subroutine entries and
// the fused lbm_step can be mixed freely.  lbm_step performs a whole time
// step as: forcing update -> fused collide+stream -> bounce-back ->
// particle update -> links -> refill, and leaves macrovar's output to be
// materialised lazily (only when something reads it).
#include <atomic>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_internal.cuh"

using namespace lbm;

namespace {

std::atomic<long long> g_launches{0};

constexpr int kStagingDoubles = 1 << 25;  // 256 MB chunk for host transfers

struct ForceState {
  int mode;  // FM_NONE / FM_TABLE / FM_CONST
  int slot;  // table slot for FM_TABLE
};

}  // namespace

struct lbm_ctx {
  lbm_config cfg;
  Geometry g;
  Rates r;
  PartParams pp;
  bool f32 = false;
  size_t esz = 8;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // next step's FORCING, launched early on a side stream (see do_forcing)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_main = nullptr, ev_forcing = nullptr, ev_status = nullptr;
  // particle work of a fused step that needs no post-collision populations
  // (the new flag buffer's reset, beads_lubforce) runs here beside the
  // bounce-back (particle_phase)
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_aux_fork = nullptr, ev_aux_join = nullptr, ev_store = nullptr;
  bool aux_pending = false;
  bool store_pending = false;  // the bounce-back stores run on aux until ev_store
  bool prefetched = false;
  int prefetch_slot = 0;
  ForcingDev* d_forcing_backup = nullptr;
  bool status_pending = false;
  std::string err;

  void* f[2] = {nullptr, nullptr};
  int cur = 0;
  void* macro = nullptr;  // rho, ux, uy, uz (4*N of T)
  bool macro_pending = false;  // macrovar of the current f not yet materialised
  bool macro_derived = true;   // macro arrays equal macrovar(f) (or pending)
  int32_t* flags[2] = {nullptr, nullptr};
  int fcur = 0;
  // statistics work space (cuFFT plans, shell permutation), made on first use
  SpectrumWork* spec = nullptr;
  // member of an lbm_batch (stepped only through the batch); batch_ready:
  // the next step's FORCING already ran, into slot batch_slot
  bool in_batch = false;
  bool batch_ready = false;
  int batch_slot = 0;
  // stream + collide kernel (lbm_set_variant / lbm_autotune)
  int variant = LBM_VARIANT_DIRECT;
  StagedPlan staged;
  // arithmetic of the FP64 collision (lbm_set_sums)
  int sums = LBM_SUMS_FLOAT;
  // FP64 fixed-point direct kernel: this step's body force per node (3 x N),
  // kept for the next step's macroscopic velocity.  It holds the field of
  // table slot fcache_slot as that slot stood at version fcache_version;
  // every (re)write of a slot bumps its version.
  double* fcache = nullptr;
  int fcache_slot = -1;
  unsigned long long fcache_version = 0;
  unsigned long long slot_version[3] = {0, 0, 0};

  // forcing
  ForcingDev* d_forcing = nullptr;
  double* d_kxr6 = nullptr;
  double* d_kyr5 = nullptr;
  double* d_kzr5 = nullptr;
  void* ztab = nullptr;  // (kx, z) partial sums of the force series, population precision
  void* ytw = nullptr;   // (cos, sin) of 2 pi ky y / ny, [5][ny], population precision
  double* ztw = nullptr;  // (cos, sin) of 2 pi kz z / nz, [5][nz]
  void* rowtab[3] = {nullptr, nullptr, nullptr};
  long long* rowtab_i[3] = {nullptr, nullptr, nullptr};  // FP64: coefficients in fixed point
  long long* xtw_i = nullptr;                            // FP64: twiddles in fixed point
  void* xtw = nullptr;
  ForceState latest{FM_NONE, 0}, fmacro{FM_NONE, 0};
  double var = 0, tf = 0, pi2 = 0;

  // particles
  int npmax = 0, npart = 0;
  bool particles_on = false;
  double* pbuf = nullptr;  // 15 vectors of 3*npmax
  double *ypglb, *ypglbp, *wp, *wpp, *omgp, *omgpp, *dwdt, *domgdt, *forcep, *forcepp, *torqp,
      *torqpp, *thetap, *fHIp, *flubp;
  int* first_move = nullptr;
  LinkSlab links{};
  FillList fill{};

  DevStatus* status = nullptr;
  DevStatus* status_host = nullptr;
  double* staging = nullptr;
  double* partial = nullptr;
  double* partial_host = nullptr;

  // per-phase timing (lbm_profile)
  bool prof_on = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  struct Interval { int phase; size_t e0, e1; };
  std::vector<Interval> intervals;
  size_t open_ev = 0;
};

namespace lbm {
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
}

namespace {

int fail(lbm_ctx* c, int code, const std::string& m) {
  if (c) c->err = m;
  return code;
}

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return fail(ctx, LBM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

cudaEvent_t next_event(lbm_ctx* c, size_t* idx) {
  if (c->ev_used == c->ev_pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    c->ev_pool.push_back(e);
  }
  *idx = c->ev_used;
  return c->ev_pool[c->ev_used++];
}
void prof_begin(lbm_ctx* c) {
  if (!c->prof_on) return;
  cudaEventRecord(next_event(c, &c->open_ev), c->stream);
}
void prof_end(lbm_ctx* c, int phase) {
  if (!c->prof_on) return;
  size_t e1;
  cudaEventRecord(next_event(c, &e1), c->stream);
  c->intervals.push_back({phase, c->open_ev, e1});
}

ParticleView pview(lbm_ctx* c) {
  ParticleView v;
  v.npart = c->npart;
  v.cap = c->links.cap;
  v.rad = c->cfg.rad;
  v.rhopart = c->cfg.rhopart;
  v.ypglb = c->ypglb;
  v.wp = c->wp;
  v.omgp = c->omgp;
  return v;
}

MoveState mstate(lbm_ctx* c) {
  MoveState m;
  m.ypglb = c->ypglb; m.ypglbp = c->ypglbp; m.ypold = nullptr;
  m.wp = c->wp; m.wpp = c->wpp; m.omgp = c->omgp; m.omgpp = c->omgpp;
  m.dwdt = c->dwdt; m.domgdt = c->domgdt; m.forcep = c->forcep; m.forcepp = c->forcepp;
  m.torqp = c->torqp; m.torqpp = c->torqpp; m.thetap = c->thetap; m.fHIp = c->fHIp;
  m.flubp = c->flubp; m.first_move = c->first_move;
  return m;
}

template <typename T>
ForceView<T> fview(lbm_ctx* c, const ForceState& s) {
  ForceView<T> v;
  v.mode = s.mode;
  v.rowtab = s.mode == FM_TABLE ? static_cast<const T*>(c->rowtab[s.slot]) : nullptr;
  v.xtw = static_cast<const T*>(c->xtw);
  if (!c->f32) {
    v.rowtab_i = s.mode == FM_TABLE ? c->rowtab_i[s.slot] : nullptr;
    v.xtw_i = c->xtw_i;
  }
  v.cfx = T(0);
  v.cfy = T(c->cfg.force_y);
  v.cfz = T(0);
  return v;
}

// The FP64 plain path keeps the current populations in 64-bit fixed point
// between its fused steps (g.pop_fixed; lbm_collide.cuh): its collision then
// loads and stores the integers it computes with.  Every other use of the
// current buffer goes through fbuf, which converts it back to FP64 first.
void pop_format(lbm_ctx* c, bool fixed) {
  if ((c->g.pop_fixed != 0) == fixed || c->f32) return;
  launch_pop_format(static_cast<double*>(c->f[c->cur]), 19 * c->g.N, fixed, c->status, c->stream);
  c->g.pop_fixed = fixed ? 1 : 0;
}
// the fused steps that run on fixed-point populations: FP64, fixed-point
// sums, the direct stream + collide kernel
bool fixed_path(const lbm_ctx* c) {
  // (a constant body force must fit the fixed-point force range, |F| < 2^-7)
  return !c->f32 && c->sums != LBM_SUMS_FLOAT && c->variant == LBM_VARIANT_DIRECT &&
         std::fabs(c->cfg.force_y) < 0.0078125;
}
template <typename T>
T* fbuf(lbm_ctx* c, int i) {
  if (i == c->cur && c->g.pop_fixed) pop_format(c, false);
  return static_cast<T*>(c->f[i]);
}
// the buffer as stored (the fused fixed-point step)
template <typename T>
T* fraw(lbm_ctx* c, int i) { return static_cast<T*>(c->f[i]); }
template <typename T>
T* mbuf(lbm_ctx* c, int comp) { return static_cast<T*>(c->macro) + comp * c->g.N; }

// a flag buffer: N particle ids, then the solid mask (Geometry::sw words a row)
size_t flag_bytes(const Geometry& g) {
  return (size_t)g.N * sizeof(int32_t) + (size_t)g.ny * g.nz * g.sw * sizeof(uint32_t);
}
// all nodes fluid: ids -1, mask clear
cudaError_t reset_flags_on(lbm_ctx* c, int i, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(c->flags[i], 0xff, (size_t)c->g.N * sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  return cudaMemsetAsync(c->flags[i] + c->g.N, 0,
                         (size_t)c->g.ny * c->g.nz * c->g.sw * sizeof(uint32_t), st);
}
cudaError_t reset_flags(lbm_ctx* c, int i) { return reset_flags_on(c, i, c->stream); }

// ranpp / ranff: Numerical Recipes ran1 (Park-Miller with Bays-Durham
// shuffle) as B/partlib.f90:83-115 states it
struct Ran1 {
  int32_t idum, iy = 0, iv[32] = {0};
  explicit Ran1(int seed) : idum(-std::abs(seed)) {}
  double operator()() {
    const int32_t IA = 16807, IM = 2147483647, IQ = 127773, IR = 2836, NTAB = 32;
    const int32_t NDIV = 1 + (IM - 1) / NTAB;
    if (idum <= 0 || iy == 0) {
      idum = std::max(-idum, 1);
      for (int j = NTAB + 8; j >= 1; --j) {
        const int32_t k = idum / IQ;
        idum = IA * (idum - k * IQ) - IR * k;
        if (idum < 0) idum += IM;
        if (j <= NTAB) iv[j - 1] = idum;
      }
      iy = iv[0];
    }
    const int32_t k = idum / IQ;
    idum = IA * (idum - k * IQ) - IR * k;
    if (idum < 0) idum += IM;
    const int32_t j = iy / NDIV;
    iy = iv[j];
    iv[j] = idum;
    return std::min((1.0 / IM) * (double)iy, 1.0 - 1.2e-7);
  }
};

// initpartpos (B/partlib.f90:1-80, C/partlib.f90:10-24): uniform centres,
// every particle that comes within mingap of a later one drawn again
// (ovlpchk with istep00 = 0, B/partlib.f90:118-171); y is (3, npart).
// Same draws and same overlap flags as the reference's all-pairs test, which
// this restricts, per round, to the pairs that can have changed: a pair of
// particles that both kept their place tested clear in the round before, so
// only a particle drawn again is tested, against the particles in its own
// and the neighbouring cells of a grid whose cells are at least the overlap
// distance 2 rad + mingap wide.  Each candidate pair is tested with the
// reference's own expression (nearest image, distance minus 2 rad + mingap).
// The cost of a round falls from npart^2 / 2 tests to (particles drawn
// again) x (neighbours); near the densest packings the algorithm reaches,
// placements take thousands of rounds with a handful of particles each.
bool init_particle_positions(const Geometry& g, int npart, double rad, double mingap,
                             double mingap_w, int seed, int max_rounds, double* y) {
  Ran1 rng(seed);
  const double radpgap = rad + mingap_w;
  auto near = [](double c, double p, int n, int nh) {
    if (c - p > nh) c -= n;
    if (c - p < -nh) c += n;
    return c;
  };
  // the reference's test of particle a against a later particle b
  auto overlap = [&](int a, int b) {
    const double xc = y[3 * a], yc = y[3 * a + 1], zc = y[3 * a + 2];
    double xb = y[3 * b], yb = y[3 * b + 1], zb = y[3 * b + 2];
    if (!g.channel) xb = near(xb, xc, g.nx, g.nxh);
    yb = near(yb, yc, g.ny, g.nyh);
    zb = near(zb, zc, g.nz, g.nzh);
    const double dx = xc - xb, dy = yc - yb, dz = zc - zb;
    return std::sqrt(dx * dx + dy * dy + dz * dz) - 2.0 * rad - mingap < 0.0;
  };
  const int ext[3] = {g.nx, g.ny, g.nz};
  const bool periodic[3] = {!g.channel, true, true};
  const double cut = 2.0 * rad + mingap;
  int nc[3];
  double inv[3];
  for (int a = 0; a < 3; ++a) {
    // cells of at least the overlap distance (with a margin for its
    // rounding); with fewer than three cells on an axis the neighbours
    // would coincide, so that axis has one cell
    int c = cut > 0.0 ? (int)std::floor((double)ext[a] / (cut * 1.0001)) : 1;
    if (c < 3) c = 1;
    nc[a] = c;
    inv[a] = (double)c / (double)ext[a];
  }
  auto coord = [&](int i, int a) {
    const int k = (int)(y[3 * i + a] * inv[a]);
    return k < 0 ? 0 : (k >= nc[a] ? nc[a] - 1 : k);
  };
  auto cell_of = [&](int i) { return coord(i, 0) + nc[0] * (coord(i, 1) + nc[1] * coord(i, 2)); };
  std::vector<std::vector<int>> members((size_t)nc[0] * nc[1] * nc[2]);
  std::vector<int> cell(npart, -1), moved, flagged;
  std::vector<char> is_moved(npart, 0), flag(npart, 0);
  for (int i = 0; i < npart; ++i) moved.push_back(i);
  for (int round = 0; round < max_rounds; ++round) {
    for (int ip : moved) {  // in index order, as the reference draws
      y[3 * ip] = g.channel ? radpgap + ((double)g.nx - 2.0 * radpgap) * rng() : (double)g.nx * rng();
      y[3 * ip + 1] = (double)g.ny * rng();
      y[3 * ip + 2] = (double)g.nz * rng();
      const int c = cell_of(ip);
      if (c != cell[ip]) {
        if (cell[ip] >= 0) {
          std::vector<int>& v = members[cell[ip]];
          v.erase(std::find(v.begin(), v.end(), ip));
        }
        members[c].push_back(ip);
        cell[ip] = c;
      }
      is_moved[ip] = 1;
    }
    flagged.clear();
    for (int r : moved) {
      int nb[3][3], nn[3];
      for (int a = 0; a < 3; ++a) {
        nn[a] = 0;
        const int cr = coord(r, a);
        if (nc[a] == 1) {
          nb[a][nn[a]++] = 0;
          continue;
        }
        for (int d = -1; d <= 1; ++d) {
          int c = cr + d;
          if (periodic[a]) c = (c + nc[a]) % nc[a];
          else if (c < 0 || c >= nc[a]) continue;
          nb[a][nn[a]++] = c;
        }
      }
      for (int iz = 0; iz < nn[2]; ++iz)
        for (int iy = 0; iy < nn[1]; ++iy)
          for (int ix = 0; ix < nn[0]; ++ix)
            for (int q : members[nb[0][ix] + nc[0] * (nb[1][iy] + nc[1] * nb[2][iz])]) {
              if (q == r || (is_moved[q] && q < r)) continue;  // each pair once
              const int a = q < r ? q : r, b = q < r ? r : q;
              if (!flag[a] && overlap(a, b)) {
                flag[a] = 1;
                flagged.push_back(a);
              }
            }
    }
    for (int r : moved) is_moved[r] = 0;
    std::sort(flagged.begin(), flagged.end());
    for (int a : flagged) flag[a] = 0;
    moved.swap(flagged);
    if (moved.empty()) return true;
  }
  return false;
}

int check_status(lbm_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->status_host, ctx->status, sizeof(DevStatus), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  DevStatus s = *ctx->status_host;
  if (s.code != 0) {
    CK(cudaMemsetAsync(ctx->status, 0, sizeof(DevStatus), ctx->stream));
    char buf[160];
    const char* what = s.code == LBM_ERR_OVERLAP    ? "particles overlap after a move"
                       : s.code == LBM_ERR_CAPACITY ? "link or geometry capacity exceeded"
                       : s.code == LBM_ERR_STATE    ? "particle image sweep not at a fixed point"
                       : s.code == LBM_ERR_NONFINITE ? "non-finite particle centre"
                       : s.code == LBM_ERR_TIMEOUT  ? "a bounded device-side wait ran out"
                                                    : "device error";
    snprintf(buf, sizeof buf, "%s (%s %d)", what, s.code == LBM_ERR_TIMEOUT ? "block" : "particle",
             s.where);
    return fail(ctx, s.code, buf);
  }
  return 0;
}

template <typename T>
void materialize_macro_t(lbm_ctx* c) {
  launch_macrovar<T>(c->g, fbuf<T>(c, c->cur), c->flags[c->fcur], fview<T>(c, c->fmacro),
                     pview(c), mbuf<T>(c, 0), mbuf<T>(c, 1), mbuf<T>(c, 2), mbuf<T>(c, 3),
                     c->stream);
}
void materialize_macro(lbm_ctx* c) {
  if (!c->macro_pending) return;
  if (c->f32) materialize_macro_t<float>(c); else materialize_macro_t<double>(c);
  c->macro_pending = false;
  c->macro_derived = true;
}

int pick_slot(lbm_ctx* c) {
  for (int s = 0; s < 3; ++s) {
    bool used = (c->latest.mode == FM_TABLE && c->latest.slot == s) ||
                (c->fmacro.mode == FM_TABLE && c->fmacro.slot == s);
    if (!used) return s;
  }
  return 0;
}

void launch_forcing_into(lbm_ctx* c, int slot, cudaStream_t st) {
  ++c->slot_version[slot];
  launch_forcing_update(c->d_forcing, c->var, c->tf, c->pi2, c->d_kxr6, c->d_kyr5, c->d_kzr5, st);
  if (c->f32)
    launch_forcing_tables<float>(c->g, c->d_forcing, static_cast<const float*>(c->ytw), c->ztw,
                                 static_cast<float*>(c->rowtab[slot]),
                                 static_cast<float*>(c->ztab), st);
  else
    launch_forcing_tables<double>(c->g, c->d_forcing, static_cast<const double*>(c->ytw),
                                  c->ztw, static_cast<double*>(c->rowtab[slot]),
                                  static_cast<double*>(c->ztab), st, c->rowtab_i[slot], c->status);
}

// FORCING: advance the stochastic state and tabulate the new field.  If the
// previous lbm_step already launched this call on the side stream, it is
// consumed here (the main stream waits for it).
void do_forcing(lbm_ctx* c) {
  if (c->cfg.forcing == LBM_FORCING_STOCHASTIC) {
    if (c->prefetched) {
      cudaStreamWaitEvent(c->stream, c->ev_forcing, 0);
      c->latest = {FM_TABLE, c->prefetch_slot};
      c->prefetched = false;
      return;
    }
    prof_begin(c);
    int s = pick_slot(c);
    launch_forcing_into(c, s, c->stream);
    c->latest = {FM_TABLE, s};
    prof_end(c, LBM_PHASE_FORCING);
  } else if (c->cfg.forcing == LBM_FORCING_CONSTANT) {
    c->latest = {FM_CONST, 0};
  } else {
    c->latest = {FM_NONE, 0};
  }
}

// Launch the next step's FORCING on the side stream, right after this step's
// FORCING was taken (do_forcing): it runs beside this step's stream +
// collide, whose FP64 fixed-point and FP32 kernels leave the FP64 pipe idle,
// rather than beside the particle kernels, which need that pipe (this GPU
// issues FP64 at 2 lanes per clock per SM).  The forcing state is backed up
// first so that cancel_prefetch can undo it.
void prefetch_forcing(lbm_ctx* c) {
  if (c->cfg.forcing != LBM_FORCING_STOCHASTIC || c->prefetched) return;
  // the slot neither this step's force nor the previous one's (macrovar's)
  // occupies: its last reader is the previous step's stream + collide
  const int slot = pick_slot(c);
  cudaEventRecord(c->ev_main, c->stream);
  cudaStreamWaitEvent(c->side, c->ev_main, 0);
  cudaMemcpyAsync(c->d_forcing_backup, c->d_forcing, sizeof(ForcingDev), cudaMemcpyDeviceToDevice,
                  c->side);
  if (c->prof_on) {
    size_t e0, e1;
    cudaEventRecord(next_event(c, &e0), c->side);
    launch_forcing_into(c, slot, c->side);
    cudaEventRecord(next_event(c, &e1), c->side);
    c->intervals.push_back({LBM_PHASE_FORCING, e0, e1});
  } else {
    launch_forcing_into(c, slot, c->side);
  }
  cudaEventRecord(c->ev_forcing, c->side);
  c->prefetched = true;
  c->prefetch_slot = slot;
}

// Undo a prefetched FORCING (restore the generator and OU state).
void cancel_prefetch(lbm_ctx* c) {
  if (!c->prefetched) return;
  cudaStreamWaitEvent(c->stream, c->ev_forcing, 0);
  cudaMemcpyAsync(c->d_forcing, c->d_forcing_backup, sizeof(ForcingDev), cudaMemcpyDeviceToDevice,
                  c->stream);
  c->prefetched = false;
}

// The part of the particle step that reads no post-collision populations:
// the reset of the flag buffer beads_links fills next (last read by the
// previous step's beads_filling) and beads_lubforce (positions only).  A
// fused step launches it on the aux stream right after stream + collide, so
// it runs beside the bounce-back; particle_phase joins it.
void particle_prelude(lbm_ctx* c) {
  if (!c->particles_on || c->aux_pending) return;
  cudaEventRecord(c->ev_aux_fork, c->stream);
  cudaStreamWaitEvent(c->aux, c->ev_aux_fork, 0);
  reset_flags_on(c, 1 - c->fcur, c->aux);
  launch_lubforce(c->g, c->npart, c->pp, mstate(c), c->aux);
  cudaEventRecord(c->ev_aux_join, c->aux);
  c->aux_pending = true;
}

// The bounce-back stores of a fused step (beads_collision's writes) on the
// aux stream: they must land before beads_links rewrites the link slab they
// read and before beads_filling reads populations, so beads_move and the link
// sweeps run beside them; particle_phase joins them before the links.
template <typename T>
void bounce_store_aux(lbm_ctx* c, T* fout) {
  cudaEventRecord(c->ev_aux_fork, c->stream);
  cudaStreamWaitEvent(c->aux, c->ev_aux_fork, 0);
  launch_bounce_scatter<T>(c->g, pview(c), fout, 1, c->links, c->aux, c->status);
  cudaEventRecord(c->ev_store, c->aux);
  c->store_pending = true;
}

template <typename T>
void particle_phase(lbm_ctx* c, T* f_plain) {
  // beads_lubforce, beads_move, beads_redistribute, beads_links, beads_filling
  const bool pre = c->aux_pending;
  if (pre) {
    cudaStreamWaitEvent(c->stream, c->ev_aux_join, 0);
    c->aux_pending = false;
  }
  prof_begin(c);
  if (!pre) launch_lubforce(c->g, c->npart, c->pp, mstate(c), c->stream);
  const ParticleView pv = pview(c);
  const bool ovl_aux = launch_move_redistribute(c->g, c->npart, c->pp, mstate(c), c->status,
                                                c->stream, c->aux, c->ev_aux_fork, c->ev_aux_join,
                                                &pv, &c->links);
  prof_end(c, LBM_PHASE_PARTICLES);
  int nf = 1 - c->fcur;
  prof_begin(c);
  if (!pre) reset_flags(c, nf);
  if (c->store_pending) {
    cudaStreamWaitEvent(c->stream, c->ev_store, 0);
    c->store_pending = false;
  }
  launch_links(c->g, pview(c), c->flags[nf], c->links, c->status, c->f32 ? 1 : 0, c->stream, true);
  prof_end(c, LBM_PHASE_LINKS);
  prof_begin(c);
  launch_filling<T>(c->g, pview(c), c->pp, c->ypglbp, c->wpp, c->omgpp, c->flags[nf],
                    c->flags[c->fcur], f_plain, c->fill, c->status, c->stream);
  prof_end(c, LBM_PHASE_FILLING);
  if (ovl_aux) cudaStreamWaitEvent(c->stream, c->ev_aux_join, 0);  // the overlap check
  c->fcur = nf;
}

// the fused stream + collide of the selected variant, fin -> fout.
// use_cache: a step (not a timing run) that may read and must then refresh
// the per-node force cache of the FP64 fixed-point direct kernel.
template <typename T>
void launch_stream_collide(lbm_ctx* c, const T* fin, T* fout, bool use_cache = false) {
  if (c->variant == LBM_VARIANT_STAGED || c->variant == LBM_VARIANT_STAGED_X2) {
    launch_fused_staged<T>(c->g, c->r, fin, fout, c->flags[c->fcur], fview<T>(c, c->fmacro),
                           fview<T>(c, c->latest), c->staged, c->status, c->stream);
    if (use_cache) c->fcache_slot = -1;
    return;
  }
  int mode = 0;
  const bool fx = !c->f32 && c->sums != LBM_SUMS_FLOAT;
  if (use_cache && fx && c->fcache && c->latest.mode == FM_TABLE) {
    const bool hit = c->fmacro.mode == FM_TABLE && c->fmacro.slot == c->fcache_slot &&
                     c->slot_version[c->fcache_slot] == c->fcache_version;
    mode = hit ? 2 : 1;
  }
  bool done = false;
  if constexpr (sizeof(T) == 8) {
    if (c->g.pop_fixed) {  // fin and fout in fixed point (fixed_path)
      launch_fused_fixed(c->g, c->r, c->sums == LBM_SUMS_INTEGER, fin, fout, c->flags[c->fcur],
                         fview<T>(c, c->fmacro),
                         fview<T>(c, c->latest), reinterpret_cast<T*>(c->fcache), mode,
                         c->status, c->stream);
      done = true;
    }
  }
  if (!done) {
    // the force cache holds fixed-point forces of the fixed-point kernel only
    mode = 0;
    launch_fused_step<T>(c->g, c->r, fin, fout, c->flags[c->fcur], fview<T>(c, c->fmacro),
                         fview<T>(c, c->latest), fx, reinterpret_cast<T*>(c->fcache), mode,
                         c->stream);
  }
  if (use_cache) {
    c->fcache_slot = mode ? c->latest.slot : -1;
    c->fcache_version = mode ? c->slot_version[c->latest.slot] : 0;
  }
}

// plan a staged variant with `stages` stages (0: the default, four where two
// CTAs of that size fit on an SM, else fewer) and ctas_per_sm resident CTAs
// (0: as many as fit)
bool plan_staged(lbm_ctx* c, int variant, int stages, int ctas_per_sm, StagedPlan* p,
                 int groups = 1) {
  const bool packed = variant == LBM_VARIANT_STAGED_X2;
  const bool fx = !c->f32 && c->sums != LBM_SUMS_FLOAT;
  if (variant != LBM_VARIANT_STAGED && !packed) return false;
  if (stages == 0) {
    for (int S = 4; S >= 2 && stages == 0; --S) {
      StagedPlan t;
      const bool ok = c->f32 ? plan_fused_staged<float>(c->g, S, 0, packed, groups, &t)
                             : plan_fused_staged<double>(c->g, S, 0, packed, groups, &t, fx);
      if (ok && (t.ctas_per_sm >= 2 || S == 2)) stages = S;
    }
    if (stages == 0) return false;
  }
  return c->f32 ? plan_fused_staged<float>(c->g, stages, ctas_per_sm, packed, groups, p)
                : plan_fused_staged<double>(c->g, stages, ctas_per_sm, packed, groups, p, fx);
}

template <typename T>
void fused_step_t(lbm_ctx* c) {
  do_forcing(c);
  prefetch_forcing(c);
  const bool fixed = fixed_path(c);
  if (fixed) pop_format(c, true);
  T* fin = fixed ? fraw<T>(c, c->cur) : fbuf<T>(c, c->cur);
  T* fout = fraw<T>(c, 1 - c->cur);
  prof_begin(c);
  launch_stream_collide<T>(c, fin, fout, true);
  prof_end(c, LBM_PHASE_STREAM_COLLIDE);
  particle_prelude(c);
  if (c->particles_on) {
    prof_begin(c);
    launch_bounce_back<T>(c->g, pview(c), fout, 1, c->flags[c->fcur], c->links, c->fHIp,
                          c->torqp, c->stream);
    prof_end(c, LBM_PHASE_BOUNCE);
    bounce_store_aux<T>(c, fout);
    particle_phase<T>(c, fout);
  } else {
    // without particles both flag buffers say "all fluid"; flipping keeps
    // the buffer parity the same for every box of a batch
    c->fcur = 1 - c->fcur;
  }
  c->cur = 1 - c->cur;
  c->fmacro = c->latest;
  c->macro_pending = true;
  c->macro_derived = true;
}

// the unfused sequence of main.f90:172-188, used when the stored macro
// arrays are not macrovar's output of the current populations
template <typename T>
void unfused_step_t(lbm_ctx* c) {
  materialize_macro(c);
  do_forcing(c);
  launch_collision<T>(c->g, c->r, fbuf<T>(c, c->cur), c->flags[c->fcur], fview<T>(c, c->latest),
                      mbuf<T>(c, 0), mbuf<T>(c, 1), mbuf<T>(c, 2), mbuf<T>(c, 3), c->stream);
  if (c->particles_on) {
    launch_bounce_back<T>(c->g, pview(c), fbuf<T>(c, c->cur), 0, c->flags[c->fcur], c->links,
                          c->fHIp, c->torqp, c->stream);
    launch_bounce_scatter<T>(c->g, pview(c), fbuf<T>(c, c->cur), 0, c->links, c->stream);
  }
  launch_streaming<T>(c->g, fbuf<T>(c, c->cur), fbuf<T>(c, 1 - c->cur), c->stream);
  c->cur = 1 - c->cur;
  if (c->particles_on) particle_phase<T>(c, fbuf<T>(c, c->cur));
  else c->fcur = 1 - c->fcur;  // as fused_step_t
  c->fmacro = c->latest;
  c->macro_pending = true;
  c->macro_derived = true;
}

int64_t default_link_capacity(double rad) {
  const double pi = 4.0 * std::atan(1.0);
  double ro = rad + 2.0, ri = rad > 1.0 ? rad - 1.0 : 0.0;
  double shell = 4.0 / 3.0 * pi * (ro * ro * ro - ri * ri * ri);
  int64_t cap = (int64_t)std::ceil(shell * 10.0);
  if (cap < 256) cap = 256;
  return (cap + 31) / 32 * 32;
}

uint64_t footprint(const lbm_config& c, int64_t* cap_out) {
  uint64_t N = (uint64_t)c.nx * c.ny * c.nz;
  uint64_t es = c.precision == LBM_PREC_F32 ? 4 : 8;
  uint64_t b = 0;
  b += 2 * 19 * N * es;   // populations
  b += 4 * N * es;        // macro
  b += 2 * (N * 4 + (uint64_t)c.ny * c.nz * 16 * ((c.nx + 127) / 128));  // flags + masks
  uint64_t np = c.npart_max > 0 ? c.npart_max : 0;
  int64_t cap = c.link_capacity > 0 ? c.link_capacity : default_link_capacity(c.rad);
  if (cap_out) *cap_out = cap;
  b += np * 15 * 3 * 8;
  b += np * (uint64_t)cap * (4 + 8 + 8) + np * 4;
  b += np * (kSweepBytes + 3 * 4);                       // nearest-image sweeps
  if (np > 0) b += 2ull * std::max<uint64_t>(4096, 256 * np) * 4 + 4;  // refill list
  if (c.forcing == LBM_FORCING_STOCHASTIC) {
    b += 3ull * kRowCoef * c.ny * c.nz * es + 45ull * c.nz * 2 * 8;  // row tables, z table
    b += 10ull * (c.ny + c.nz) * 8 + 2 * sizeof(ForcingDev) + 32 * 8;
    if (c.precision != LBM_PREC_F32) {
      b += 3 * N * 8;                              // per-node force cache
      b += 3ull * kRowCoef * c.ny * c.nz * 8;      // row tables in fixed point
    }
  }
  b += 4ull * c.nx * es;
  if (c.precision != LBM_PREC_F32) b += 4ull * c.nx * 8;  // twiddles in fixed point
  uint64_t stage = std::min<uint64_t>(19 * N, kStagingDoubles) * 8;
  b += stage;
  return b;
}

// Device address of a host buffer the GPU can read and write directly:
// page-locked memory (cudaHostAlloc, cudaHostRegister).  Pageable memory
// gives nullptr and takes the staged path.
const void* mapped_host(const void* h) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

template <typename T>
int upload_soa_t(lbm_ctx* ctx, const double* h, bool aos) {
  const long long N = ctx->g.N;
  T* f = fbuf<T>(ctx, ctx->cur);
  const double* hm = aos ? static_cast<const double*>(mapped_host(h)) : nullptr;
  if (hm) {
    // one pass over the link: the kernel reads the host array in place
    launch_aos_host_to_soa<T>(hm, f, N, sm_count(), ctx->stream);
  } else if (aos) {
    long long chunk = kStagingDoubles / 19;
    for (long long n0 = 0; n0 < N; n0 += chunk) {
      long long nn = std::min(chunk, N - n0);
      CK(cudaMemcpyAsync(ctx->staging, h + n0 * 19, nn * 19 * sizeof(double),
                         cudaMemcpyHostToDevice, ctx->stream));
      launch_aos_to_soa<T>(ctx->g, ctx->staging, f, n0, nn, ctx->stream);
    }
  } else if (!ctx->f32) {
    CK(cudaMemcpyAsync(f, h, 19 * N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  } else {
    long long total = 19 * N;
    for (long long o = 0; o < total; o += kStagingDoubles) {
      long long nn = std::min<long long>(kStagingDoubles, total - o);
      CK(cudaMemcpyAsync(ctx->staging, h + o, nn * sizeof(double), cudaMemcpyHostToDevice,
                         ctx->stream));
      launch_convert<T>(ctx->staging, f + o, nn, ctx->stream);
    }
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return 0;
}

template <typename T>
int download_soa_t(lbm_ctx* ctx, double* h, bool aos) {
  const long long N = ctx->g.N;
  double* hm = aos ? static_cast<double*>(const_cast<void*>(mapped_host(h))) : nullptr;
  if constexpr (sizeof(T) == 8) {
    if (hm && ctx->g.pop_fixed) {
      // page-locked host array: convert from the fixed point on the way out,
      // leaving the stored populations (and the next fused step) as they are
      launch_soa_fixed_to_aos_host(reinterpret_cast<const long long*>(fraw<T>(ctx, ctx->cur)), hm,
                                   N, sm_count(), ctx->stream);
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(ctx->stream));
      return 0;
    }
  }
  T* f = fbuf<T>(ctx, ctx->cur);
  if (hm) {
    launch_soa_to_aos_host<T>(f, hm, N, sm_count(), ctx->stream);
  } else if (aos) {
    long long chunk = kStagingDoubles / 19;
    for (long long n0 = 0; n0 < N; n0 += chunk) {
      long long nn = std::min(chunk, N - n0);
      launch_soa_to_aos<T>(ctx->g, f, ctx->staging, n0, nn, ctx->stream);
      CK(cudaMemcpyAsync(h + n0 * 19, ctx->staging, nn * 19 * sizeof(double),
                         cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
    }
  } else if (!ctx->f32) {
    CK(cudaMemcpyAsync(h, f, 19 * N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  } else {
    long long total = 19 * N;
    for (long long o = 0; o < total; o += kStagingDoubles) {
      long long nn = std::min<long long>(kStagingDoubles, total - o);
      launch_convert_back<T>(f + o, ctx->staging, nn, ctx->stream);
      CK(cudaMemcpyAsync(h + o, ctx->staging, nn * sizeof(double), cudaMemcpyDeviceToHost,
                         ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
    }
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return 0;
}

// copy a host double array of n values into T device array (via staging)
template <typename T>
int h2d_field(lbm_ctx* ctx, const double* h, T* d, long long n) {
  for (long long o = 0; o < n; o += kStagingDoubles) {
    long long nn = std::min<long long>(kStagingDoubles, n - o);
    CK(cudaMemcpyAsync(ctx->staging, h + o, nn * sizeof(double), cudaMemcpyHostToDevice,
                       ctx->stream));
    launch_convert<T>(ctx->staging, d + o, nn, ctx->stream);
  }
  return 0;
}
template <typename T>
int d2h_field(lbm_ctx* ctx, const T* d, double* h, long long n) {
  for (long long o = 0; o < n; o += kStagingDoubles) {
    long long nn = std::min<long long>(kStagingDoubles, n - o);
    launch_convert_back<T>(d + o, ctx->staging, nn, ctx->stream);
    CK(cudaMemcpyAsync(h + o, ctx->staging, nn * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return 0;
}

}  // namespace

// ===========================================================================
extern "C" {

int lbm_version(void) { return 1; }

int lbm_config_init(lbm_config* cfg, int preset, int nx, int ny, int nz, int npart, double rad,
                    double rhopart) {
  if (!cfg || nx < 4 || ny < 4 || nz < 4 || npart < 0) return LBM_ERR_ARG;
  std::memset(cfg, 0, sizeof(*cfg));
  const double pi = 4.0 * std::atan(1.0);
  cfg->nx = nx; cfg->ny = ny; cfg->nz = nz;
  cfg->npart_max = npart;
  cfg->precision = LBM_PREC_F64;
  cfg->iseedf = 232300;                 // B/para.f90:20
  cfg->iseedp = 12345;                  // B/para.f90:247
  cfg->visc = 0.0036;
  cfg->rho0 = 1.0;
  cfg->rhopart = rhopart;
  cfg->rad = rad;
  cfg->mingap = 2.0;
  cfg->mingap_w = 2.0;
  cfg->vscale = 2.037183272e-3;         // B/para.f90:37
  cfg->stf0 = 0.025; cfg->stf1 = 0.002; // B/para.f90:244-245
  cfg->stf0_w = 0.025; cfg->stf1_w = 0.002;
  const double volp = 4.0 / 3.0 * pi * (rad * rad * rad);
  if (preset == LBM_PRESET_BOX) {
    cfg->mrt_type = 1;                  // B/para.f90:96
    cfg->boundary = LBM_BC_PERIODIC;
    cfg->forcing = LBM_FORCING_STOCHASTIC;
    const double gscale = 10000.0 / 4.0;  // B/para.f90:237
    cfg->fpc = volp * cfg->rho0 * 9.8 / gscale;
    const double rhog = 0.0;              // B/para.f90:239
    cfg->body_force_y = -(volp * rhog);
  } else if (preset == LBM_PRESET_CHANNEL) {
    cfg->mrt_type = 2;                  // C/para.f90:67
    cfg->boundary = LBM_BC_XWALLS;
    cfg->forcing = LBM_FORCING_CONSTANT;
    const double Rstar = 180.0;         // C/para.f90:14-19
    const double ustar = 2.0 * Rstar * cfg->visc / (double)nx;
    const double force_in_y = 2. * cfg->rho0 * ustar * ustar / (double)nx;
    const double ystar = cfg->visc / ustar;
    const double force_mag = 1.0;
    cfg->force_y = force_in_y * force_mag;
    const double g_lbm = ustar * ustar / ystar;
    cfg->fpc = volp * cfg->rho0 * g_lbm;
    cfg->body_force_y = volp * force_in_y;  // C/partlib.f90:2409
  } else {
    return LBM_ERR_ARG;
  }
  return LBM_OK;
}

int lbm_get_config(const lbm_ctx* ctx, lbm_config* cfg) {
  if (!ctx || !cfg) return LBM_ERR_ARG;
  *cfg = ctx->cfg;
  return LBM_OK;
}

int lbm_particle_count(const lbm_ctx* ctx, int* npart) {
  if (!ctx || !npart) return LBM_ERR_ARG;
  *npart = ctx->npart;
  return LBM_OK;
}

int lbm_footprint(const lbm_config* cfg, uint64_t* bytes) {
  if (!cfg || !bytes) return LBM_ERR_ARG;
  *bytes = footprint(*cfg, nullptr);
  return LBM_OK;
}

const char* lbm_last_error(const lbm_ctx* ctx) {
  if (!ctx) return "null context";
  return ctx->err.c_str();
}

int lbm_create(const lbm_config* cfg, lbm_ctx** out) {
  if (!cfg || !out) return LBM_ERR_ARG;
  *out = nullptr;
  if (cfg->nx < 4 || cfg->ny < 4 || cfg->nz < 4) return LBM_ERR_ARG;
  if ((long long)cfg->nx * cfg->ny * cfg->nz >= (1LL << 26)) return LBM_ERR_ARG;  // link code
  if (cfg->precision != LBM_PREC_F64 && cfg->precision != LBM_PREC_F32) return LBM_ERR_ARG;
  if (cfg->boundary != LBM_BC_PERIODIC && cfg->boundary != LBM_BC_XWALLS) return LBM_ERR_ARG;
  if (cfg->mrt_type < 1 || cfg->mrt_type > 3) return LBM_ERR_ARG;
  if (cfg->npart_max > 0 && !(cfg->rad > 0.0)) return LBM_ERR_ARG;
  if (cfg->forcing == LBM_FORCING_STOCHASTIC && (cfg->ny < 6 || cfg->nz < 6)) return LBM_ERR_ARG;
  lbm_ctx* ctx = new lbm_ctx();
  ctx->cfg = *cfg;
  Geometry& g = ctx->g;
  g.nx = cfg->nx; g.ny = cfg->ny; g.nz = cfg->nz;
  g.nxh = g.nx / 2; g.nyh = g.ny / 2; g.nzh = g.nz / 2;
  g.N = (long long)g.nx * g.ny * g.nz;
  g.channel = cfg->boundary == LBM_BC_XWALLS;
  g.sw = 4 * ((g.nx + 127) / 128);
  ctx->f32 = cfg->precision == LBM_PREC_F32;
  ctx->sums = ctx->f32 ? LBM_SUMS_FLOAT : LBM_SUMS_INTEGER;
  ctx->esz = ctx->f32 ? 4 : 8;
  // MRT rates, B/para.f90:91-135
  const double tau = 3.0 * cfg->visc + 0.5;
  Rates& r = ctx->r;
  if (cfg->mrt_type == 1) { r.omegepsl = 0.0; r.omegepslj = -475.0 / 63.0; r.omegxx = 0.0; }
  else { r.omegepsl = 3.0; r.omegepslj = -11.0 / 2.0; r.omegxx = -1.0 / 2.0; }
  r.s9 = 1.0 / tau; r.s13 = r.s9;
  if (cfg->mrt_type == 1) { r.s1 = 1.19; r.s2 = 1.4; r.s4 = 1.2; r.s10 = 1.4; r.s16 = 1.98; }
  else if (cfg->mrt_type == 2) { r.s1 = r.s9; r.s2 = r.s9; r.s4 = r.s9; r.s10 = r.s9; r.s16 = r.s9; }
  else { r.s1 = 1.8; r.s2 = r.s1; r.s4 = r.s9; r.s10 = r.s1; r.s16 = r.s1; }
  const double pi = 4.0 * std::atan(1.0);
  const double volp = 4.0 / 3.0 * pi * (cfg->rad * cfg->rad * cfg->rad);
  PartParams& pp = ctx->pp;
  pp.rad = cfg->rad; pp.mingap = cfg->mingap; pp.mingap_w = cfg->mingap_w; pp.fpc = cfg->fpc;
  pp.stf0 = cfg->stf0; pp.stf1 = cfg->stf1; pp.stf0_w = cfg->stf0_w; pp.stf1_w = cfg->stf1_w;
  pp.body_force_y = cfg->body_force_y;
  pp.amp = cfg->rhopart * volp;
  pp.aip = 0.4 * pp.amp * (cfg->rad * cfg->rad);
  pp.rho0 = cfg->rho0; pp.rhopart = cfg->rhopart;
  ctx->pi2 = 2.0 * pi;
  const double tscale = ctx->pi2 * cfg->vscale / (double)g.ny;  // B/para.f90:60
  ctx->var = 447.31 * ((cfg->vscale * tscale) * (cfg->vscale * tscale));  // gaussian.f90:197
  ctx->tf = 0.038 / tscale;

  int rc = 0;
  auto al = [&](void** p, size_t bytes) -> bool {
    if (rc) return false;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
      rc = fail(ctx, LBM_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
      return false;
    }
    return true;
  };
  const long long N = g.N;
  // The engine's own stream at the greatest priority: the block scheduler
  // then prefers the critical path (stream + collide, bounce-back, move,
  // links, filling) over the side and aux streams' kernels (forcing,
  // lubrication, overlap check, bounce-back stores), which have slack.
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  if (cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, prio_greatest) != cudaSuccess) {
    delete ctx;
    return LBM_ERR_CUDA;
  }
  ctx->own_stream = true;
  if (cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_aux_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_aux_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_store, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_main, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_forcing, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_status, cudaEventDisableTiming) != cudaSuccess) {
    lbm_destroy(ctx);
    return LBM_ERR_CUDA;
  }
  al(&ctx->f[0], 19 * N * ctx->esz);
  al(&ctx->f[1], 19 * N * ctx->esz);
  al(&ctx->macro, 4 * N * ctx->esz);
  al((void**)&ctx->flags[0], flag_bytes(g));
  al((void**)&ctx->flags[1], flag_bytes(g));
  al((void**)&ctx->status, sizeof(DevStatus));
  al((void**)&ctx->staging, std::min<long long>(19 * N, kStagingDoubles) * sizeof(double));
  al((void**)&ctx->partial, 6 * 1024 * sizeof(double));
  al(&ctx->xtw, 4 * g.nx * ctx->esz);
  if (!ctx->f32) al((void**)&ctx->xtw_i, 4 * g.nx * sizeof(long long));
  if (!rc && cudaMallocHost((void**)&ctx->status_host, sizeof(DevStatus)) != cudaSuccess)
    rc = fail(ctx, LBM_ERR_NOMEM, "cudaMallocHost");
  if (!rc && cudaMallocHost((void**)&ctx->partial_host, 4 * 1024 * sizeof(double)) != cudaSuccess)
    rc = fail(ctx, LBM_ERR_NOMEM, "cudaMallocHost");
  if (cfg->forcing == LBM_FORCING_STOCHASTIC) {
    al((void**)&ctx->d_forcing, sizeof(ForcingDev));
    al((void**)&ctx->d_forcing_backup, sizeof(ForcingDev));
    al((void**)&ctx->d_kxr6, 16 * sizeof(double));
    al((void**)&ctx->d_kyr5, 8 * sizeof(double));
    al((void**)&ctx->d_kzr5, 8 * sizeof(double));
    al(&ctx->ztab, 45LL * g.nz * 2 * sizeof(double));
    al(&ctx->ytw, 5LL * g.ny * 2 * sizeof(double));
    al((void**)&ctx->ztw, 5LL * g.nz * 2 * sizeof(double));
    for (int s = 0; s < 3; ++s) al(&ctx->rowtab[s], (long long)kRowCoef * g.ny * g.nz * ctx->esz);
    if (!ctx->f32) {
      al((void**)&ctx->fcache, 3 * (size_t)g.N * sizeof(double));
      for (int s = 0; s < 3; ++s)
        al((void**)&ctx->rowtab_i[s], (long long)kRowCoef * g.ny * g.nz * sizeof(long long));
    }
  }
  ctx->npmax = cfg->npart_max > 0 ? cfg->npart_max : 0;
  if (ctx->npmax > 0) {
    int64_t cap = cfg->link_capacity > 0 ? cfg->link_capacity : default_link_capacity(cfg->rad);
    ctx->links.cap = (int)cap;
    al((void**)&ctx->pbuf, 15ULL * 3 * ctx->npmax * sizeof(double));
    al((void**)&ctx->first_move, sizeof(int));
    al((void**)&ctx->links.code, (size_t)ctx->npmax * cap * sizeof(int32_t));
    al((void**)&ctx->links.alpha, (size_t)ctx->npmax * cap * sizeof(double));
    al((void**)&ctx->links.f9, (size_t)ctx->npmax * cap * sizeof(double));
    al((void**)&ctx->links.count, (size_t)ctx->npmax * sizeof(int32_t));
    al(&ctx->links.sweeps, (size_t)ctx->npmax * kSweepBytes);
    al((void**)&ctx->links.sweep_ok, (size_t)ctx->npmax * 3 * sizeof(int32_t));
    ctx->fill.cap = std::max(4096, 256 * ctx->npmax);
    al((void**)&ctx->fill.node, (size_t)ctx->fill.cap * sizeof(int32_t));
    al((void**)&ctx->fill.part, (size_t)ctx->fill.cap * sizeof(int32_t));
    al((void**)&ctx->fill.count, sizeof(int32_t));
  }
  if (rc) {
    lbm_destroy(ctx);
    return rc;
  }
  if (ctx->npmax > 0) {
    double* b = ctx->pbuf;
    size_t v = 3 * (size_t)ctx->npmax;
    double** vecs[15] = {&ctx->ypglb, &ctx->ypglbp, &ctx->wp, &ctx->wpp, &ctx->omgp,
                         &ctx->omgpp, &ctx->dwdt, &ctx->domgdt, &ctx->forcep, &ctx->forcepp,
                         &ctx->torqp, &ctx->torqpp, &ctx->thetap, &ctx->fHIp, &ctx->flubp};
    for (int i = 0; i < 15; ++i) *vecs[i] = b + i * v;
    cudaMemsetAsync(ctx->pbuf, 0, 15 * v * sizeof(double), ctx->stream);
    cudaMemsetAsync(ctx->links.count, 0, ctx->npmax * sizeof(int32_t), ctx->stream);
    cudaMemsetAsync(ctx->first_move, 0, sizeof(int), ctx->stream);
  }
  cudaMemsetAsync(ctx->f[0], 0, 19 * N * ctx->esz, ctx->stream);
  cudaMemsetAsync(ctx->f[1], 0, 19 * N * ctx->esz, ctx->stream);
  cudaMemsetAsync(ctx->macro, 0, 4 * N * ctx->esz, ctx->stream);
  reset_flags(ctx, 0);
  reset_flags(ctx, 1);
  cudaMemsetAsync(ctx->status, 0, sizeof(DevStatus), ctx->stream);
  // x twiddles for the forcing: cos/sin of 2 pi kx x / nx, kx = 1, 2
  {
    std::vector<double> tw(4 * g.nx);
    for (int x = 0; x < g.nx; ++x) {
      for (int kx = 1; kx <= 2; ++kx) {
        long long m = ((long long)kx * x) % g.nx;
        double ang = ctx->pi2 * (double)m / (double)g.nx;
        tw[4 * x + 2 * (kx - 1)] = std::cos(ang);
        tw[4 * x + 2 * (kx - 1) + 1] = std::sin(ang);
      }
    }
    if (ctx->f32) {
      std::vector<float> twf(tw.begin(), tw.end());
      cudaMemcpy(ctx->xtw, twf.data(), twf.size() * sizeof(float), cudaMemcpyHostToDevice);
    } else {
      cudaMemcpy(ctx->xtw, tw.data(), tw.size() * sizeof(double), cudaMemcpyHostToDevice);
      // the same twiddles at 2^-kTwFix (|cos|, |sin| <= 1; exact for values
      // of 2^-8 and more)
      std::vector<long long> twi(tw.size());
      for (size_t i = 0; i < tw.size(); ++i) twi[i] = std::llround(std::ldexp(tw[i], kTwFix));
      cudaMemcpy(ctx->xtw_i, twi.data(), twi.size() * sizeof(long long), cudaMemcpyHostToDevice);
    }
  }
  if (cfg->forcing == LBM_FORCING_STOCHASTIC) {
    // wavenumbers of the 6x5x5 block, B/para.f90:260-286; state 281-286
    double kx6[16] = {0}, ky5[8] = {0}, kz5[8] = {0};
    // kxr(i) = int(i/2) for odd i and kxr(i+1) = kxr(i): 0, 0, 1, 1, 2, 2
    for (int i = 1; i <= 6; ++i) kx6[i - 1] = (double)((i - 1) / 2);
    for (int j = 1; j <= 5; ++j) {
      int jj = (j > 3) ? j + g.ny - 5 : j;
      ky5[j - 1] = (jj < g.ny / 2 + 2) ? (double)(jj - 1) : (double)(-(g.ny + 1 - jj));
      int kk = (j > 3) ? j + g.nz - 5 : j;
      kz5[j - 1] = (kk < g.nz / 2 + 2) ? (double)(kk - 1) : (double)(-(g.nz + 1 - kk));
    }
    cudaMemcpy(ctx->d_kxr6, kx6, sizeof kx6, cudaMemcpyHostToDevice);
    cudaMemcpy(ctx->d_kyr5, ky5, sizeof ky5, cudaMemcpyHostToDevice);
    cudaMemcpy(ctx->d_kzr5, kz5, sizeof kz5, cudaMemcpyHostToDevice);
    auto twid = [&](const double* k5, int n, void* dst, bool f32) {
      std::vector<double> t(10 * (size_t)n);
      for (int j = 0; j < 5; ++j)
        for (int x = 0; x < n; ++x) {
          long long m = ((long long)k5[j] * x) % n;
          if (m < 0) m += n;
          double ang = ctx->pi2 * (double)m / (double)n;
          t[2 * ((size_t)j * n + x)] = std::cos(ang);
          t[2 * ((size_t)j * n + x) + 1] = std::sin(ang);
        }
      if (f32) {
        std::vector<float> tf(t.begin(), t.end());
        cudaMemcpy(dst, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice);
      } else {
        cudaMemcpy(dst, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice);
      }
    };
    twid(ky5, g.ny, ctx->ytw, ctx->f32);
    twid(kz5, g.nz, ctx->ztw, false);
    ForcingDev st;
    std::memset(&st, 0, sizeof st);
    st.iseedf = -cfg->iseedf;
    cudaMemcpy(ctx->d_forcing, &st, sizeof st, cudaMemcpyHostToDevice);
    ctx->latest = {FM_NONE, 0};
    ctx->fmacro = {FM_NONE, 0};
  } else if (cfg->forcing == LBM_FORCING_CONSTANT) {
    ctx->latest = {FM_CONST, 0};
    ctx->fmacro = {FM_CONST, 0};
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    lbm_destroy(ctx);
    return LBM_ERR_CUDA;
  }
  {
    StagedPlan p;
    if (ctx->f32) {
      if (plan_staged(ctx, LBM_VARIANT_STAGED_X2, 0, 0, &p)) {
        ctx->variant = LBM_VARIANT_STAGED_X2;
        ctx->staged = p;
      } else if (plan_staged(ctx, LBM_VARIANT_STAGED, 0, 0, &p)) {
        ctx->variant = LBM_VARIANT_STAGED;
        ctx->staged = p;
      }
    }
    cudaGetLastError();
  }
  *out = ctx;
  return LBM_OK;
}

int lbm_destroy(lbm_ctx* ctx) {
  if (!ctx) return LBM_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->side) cudaStreamSynchronize(ctx->side);
  if (ctx->aux) cudaStreamSynchronize(ctx->aux);
  spectrum_free(ctx->spec);
  ctx->spec = nullptr;
  void* ptrs[] = {ctx->f[0], ctx->f[1], ctx->macro, ctx->flags[0], ctx->flags[1], ctx->status,
                  ctx->staging, ctx->partial, ctx->xtw, ctx->d_forcing, ctx->d_kxr6,
                  ctx->d_kyr5, ctx->d_kzr5, ctx->ztab, ctx->ytw, ctx->ztw, ctx->d_forcing_backup,
                  ctx->rowtab[0], ctx->rowtab[1],
                  ctx->rowtab[2], ctx->pbuf, ctx->first_move, ctx->links.code,
                  ctx->links.alpha, ctx->links.f9, ctx->links.count, ctx->links.sweeps,
                  ctx->links.sweep_ok, ctx->fill.node,
                  ctx->fill.part, ctx->fill.count, ctx->fcache, ctx->xtw_i,
                  ctx->rowtab_i[0], ctx->rowtab_i[1], ctx->rowtab_i[2]};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->status_host) cudaFreeHost(ctx->status_host);
  if (ctx->partial_host) cudaFreeHost(ctx->partial_host);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->side) cudaStreamDestroy(ctx->side);
  if (ctx->aux) cudaStreamDestroy(ctx->aux);
  for (cudaEvent_t e : {ctx->ev_main, ctx->ev_forcing, ctx->ev_status, ctx->ev_aux_fork,
                        ctx->ev_aux_join, ctx->ev_store})
    if (e) cudaEventDestroy(e);
  delete ctx;
  return LBM_OK;
}

int lbm_set_stream(lbm_ctx* ctx, void* stream) {
  if (!ctx) return LBM_ERR_ARG;
  cancel_prefetch(ctx);
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaStreamSynchronize(ctx->side));
  if (stream) {
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    ctx->stream = static_cast<cudaStream_t>(stream);
    ctx->own_stream = false;
  }
  return LBM_OK;
}

int lbm_synchronize(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->side));
  ctx->status_pending = false;
  return check_status(ctx);
}

int lbm_upload_f(lbm_ctx* ctx, const double* f) {
  if (!ctx || !f) return LBM_ERR_ARG;
  int rc = ctx->f32 ? upload_soa_t<float>(ctx, f, true) : upload_soa_t<double>(ctx, f, true);
  ctx->macro_pending = false;
  ctx->macro_derived = false;
  return rc;
}
int lbm_download_f(lbm_ctx* ctx, double* f) {
  if (!ctx || !f) return LBM_ERR_ARG;
  return ctx->f32 ? download_soa_t<float>(ctx, f, true) : download_soa_t<double>(ctx, f, true);
}
int lbm_upload_f_soa(lbm_ctx* ctx, const double* f) {
  if (!ctx || !f) return LBM_ERR_ARG;
  int rc = ctx->f32 ? upload_soa_t<float>(ctx, f, false) : upload_soa_t<double>(ctx, f, false);
  ctx->macro_pending = false;
  ctx->macro_derived = false;
  return rc;
}
int lbm_download_f_soa(lbm_ctx* ctx, double* f) {
  if (!ctx || !f) return LBM_ERR_ARG;
  return ctx->f32 ? download_soa_t<float>(ctx, f, false) : download_soa_t<double>(ctx, f, false);
}

// initpop from a device velocity field dv[3][N]; frees dv
static int initpop_device(lbm_ctx* ctx, double* dv) {
  const long long N = ctx->g.N;
  if (ctx->f32) {
    launch_initpop<float>(ctx->g, dv, dv + N, dv + 2 * N, fbuf<float>(ctx, ctx->cur),
                          mbuf<float>(ctx, 0), ctx->stream);
    for (int c = 0; c < 3; ++c) launch_convert<float>(dv + c * N, mbuf<float>(ctx, 1 + c), N, ctx->stream);
  } else {
    launch_initpop<double>(ctx->g, dv, dv + N, dv + 2 * N, fbuf<double>(ctx, ctx->cur),
                           mbuf<double>(ctx, 0), ctx->stream);
    cudaMemcpyAsync(mbuf<double>(ctx, 1), dv, 3 * N * sizeof(double), cudaMemcpyDeviceToDevice,
                    ctx->stream);
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  cudaFree(dv);
  if (e != cudaSuccess) return fail(ctx, LBM_ERR_CUDA, cudaGetErrorString(e));
  CK(cudaGetLastError());
  ctx->macro_pending = false;
  ctx->macro_derived = false;
  return LBM_OK;
}

int lbm_initpop(lbm_ctx* ctx, const double* ux, const double* uy, const double* uz) {
  if (!ctx || !ux || !uy || !uz) return LBM_ERR_ARG;
  const long long N = ctx->g.N;
  double* dv = nullptr;
  CK(cudaMalloc((void**)&dv, 3 * N * sizeof(double)));
  cudaMemcpyAsync(dv, ux, N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(dv + N, uy, N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(dv + 2 * N, uz, N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  return initpop_device(ctx, dv);
}

int lbm_init_spectral(lbm_ctx* ctx, double k0, double u_rms, uint64_t seed) {
  if (!ctx || !(k0 > 0.0) || u_rms < 0.0) return LBM_ERR_ARG;
  const long long N = ctx->g.N;
  double* dv = nullptr;
  CK(cudaMalloc((void**)&dv, 3 * N * sizeof(double)));
  if (int rc = spectral_field(ctx->g, k0, u_rms, seed, dv, ctx->stream)) {
    cudaFree(dv);
    cudaGetLastError();
    return fail(ctx, rc, "init_spectral: FFT or allocation failed");
  }
  return initpop_device(ctx, dv);
}

int lbm_init_channel(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  if (!ctx->g.channel) return fail(ctx, LBM_ERR_ARG, "init_channel: the box has no walls");
  const long long N = ctx->g.N;
  double* dv = nullptr;
  CK(cudaMalloc((void**)&dv, 3 * N * sizeof(double)));
  if (int rc = channel_loglaw_field(ctx->g, ctx->cfg.visc, dv, ctx->stream)) {
    cudaFree(dv);
    cudaGetLastError();
    return fail(ctx, rc, "init_channel: launch failed");
  }
  return initpop_device(ctx, dv);
}

int lbm_place_particles(const lbm_config* cfg, int npart, int seed, int max_rounds,
                        double* ypglb) {
  if (!cfg || npart < 0 || (npart > 0 && !ypglb)) return LBM_ERR_ARG;
  if (cfg->nx < 1 || cfg->ny < 1 || cfg->nz < 1 || (npart > 0 && !(cfg->rad > 0.0)))
    return LBM_ERR_ARG;
  Geometry g{};
  g.nx = cfg->nx; g.ny = cfg->ny; g.nz = cfg->nz;
  g.nxh = g.nx / 2; g.nyh = g.ny / 2; g.nzh = g.nz / 2;
  g.channel = cfg->boundary == LBM_BC_XWALLS;
  if (npart > 0 &&
      !init_particle_positions(g, npart, cfg->rad, cfg->mingap, cfg->mingap_w, seed,
                               max_rounds > 0 ? max_rounds : 100000, ypglb))
    return LBM_ERR_OVERLAP;
  return LBM_OK;
}

int lbm_init_particles(lbm_ctx* ctx, int npart, int seed, int max_rounds) {
  if (!ctx || npart < 0 || npart > ctx->npmax) return LBM_ERR_ARG;
  std::vector<double> y(3 * (size_t)npart), zero(3 * (size_t)npart, 0.0);
  if (npart > 0 &&
      !init_particle_positions(ctx->g, npart, ctx->cfg.rad, ctx->cfg.mingap, ctx->cfg.mingap_w,
                               seed, max_rounds > 0 ? max_rounds : 100000, y.data()))
    return fail(ctx, LBM_ERR_OVERLAP, "init_particles: no placement without overlap");
  return lbm_upload_particles(ctx, npart, y.data(), zero.data(), zero.data());
}

int lbm_summary(lbm_ctx* ctx, double out[6]) {
  if (!ctx || !out) return LBM_ERR_ARG;
  materialize_macro(ctx);
  const int nb = 1024;
  if (ctx->f32)
    launch_summary<float>(fbuf<float>(ctx, ctx->cur), ctx->g.N, mbuf<float>(ctx, 1),
                          mbuf<float>(ctx, 2), mbuf<float>(ctx, 3), ctx->partial, nb, ctx->stream);
  else
    launch_summary<double>(fbuf<double>(ctx, ctx->cur), ctx->g.N, mbuf<double>(ctx, 1),
                           mbuf<double>(ctx, 2), mbuf<double>(ctx, 3), ctx->partial, nb,
                           ctx->stream);
  std::vector<double> h(6 * (size_t)nb);
  CK(cudaMemcpyAsync(h.data(), ctx->partial, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int c = 0; c < 6; ++c) out[c] = 0.0;
  for (int b = 0; b < nb; ++b)
    for (int c = 0; c < 6; ++c) out[c] += h[6 * (size_t)b + c];
  return LBM_OK;
}

int lbm_download_macro(lbm_ctx* ctx, double* rho, double* ux, double* uy, double* uz) {
  if (!ctx) return LBM_ERR_ARG;
  materialize_macro(ctx);
  double* outs[4] = {rho, ux, uy, uz};
  for (int c = 0; c < 4; ++c) {
    if (!outs[c]) continue;
    int rc = ctx->f32 ? d2h_field<float>(ctx, mbuf<float>(ctx, c), outs[c], ctx->g.N)
                      : d2h_field<double>(ctx, mbuf<double>(ctx, c), outs[c], ctx->g.N);
    if (rc) return rc;
  }
  CK(cudaGetLastError());
  return LBM_OK;
}

static int poll_status(lbm_ctx* ctx);

int lbm_statistics(lbm_ctx* ctx, int nek, double* ek, double* dk, double* out) {
  if (!ctx || !out || nek < 0 || (nek > 0 && (!ek || !dk))) return LBM_ERR_ARG;
  if (int rc = poll_status(ctx)) return rc;
  materialize_macro(ctx);
  int rc = ctx->f32 ? spectrum_stats<float>(ctx->g, ctx->cfg.visc, mbuf<float>(ctx, 1),
                                            mbuf<float>(ctx, 2), mbuf<float>(ctx, 3), &ctx->spec,
                                            nek, ek, dk, out, ctx->stream)
                    : spectrum_stats<double>(ctx->g, ctx->cfg.visc, mbuf<double>(ctx, 1),
                                             mbuf<double>(ctx, 2), mbuf<double>(ctx, 3), &ctx->spec,
                                             nek, ek, dk, out, ctx->stream);
  if (rc) {
    cudaGetLastError();
    return fail(ctx, rc, "statistics: FFT or allocation failed");
  }
  CK(cudaGetLastError());
  return LBM_OK;
}

// mean and rms of one component of (3, n) particle vectors, summed in index
// order as the reference's sum() over a vector
static void part_mean_rms(const std::vector<double>& v, int n, int c, double* mn, double* rms) {
  double s = 0.0;
  for (int p = 0; p < n; ++p) s += v[3 * p + c];
  *mn = s / (double)n;
  double q = 0.0;
  for (int p = 0; p < n; ++p) q += (v[3 * p + c] - *mn) * (v[3 * p + c] - *mn);
  *rms = std::sqrt(q / (double)n);
}

int lbm_rmsstat(lbm_ctx* ctx, double* out) {
  if (!ctx || !out) return LBM_ERR_ARG;
  if (int rc = poll_status(ctx)) return rc;
  materialize_macro(ctx);
  double fl[13];
  int rc = ctx->f32 ? fluid_rms_stats<float>(ctx->g, ctx->flags[ctx->fcur], mbuf<float>(ctx, 1),
                                             mbuf<float>(ctx, 2), mbuf<float>(ctx, 3), &ctx->spec,
                                             fl, ctx->stream)
                    : fluid_rms_stats<double>(ctx->g, ctx->flags[ctx->fcur], mbuf<double>(ctx, 1),
                                              mbuf<double>(ctx, 2), mbuf<double>(ctx, 3),
                                              &ctx->spec, fl, ctx->stream);
  if (rc) {
    cudaGetLastError();
    return fail(ctx, rc, "rmsstat: FFT or allocation failed");
  }
  const double nf = fl[0];
  const double nx3 = (double)ctx->g.nx * ctx->g.nx * ctx->g.nx;  // real(nx**3), saveload.f90:1712
  double wmn[3] = {0, 0, 0}, wrms[3] = {0, 0, 0}, omn[3] = {0, 0, 0}, orms[3] = {0, 0, 0};
  const int np = ctx->particles_on ? ctx->npart : 0;
  if (np > 0) {
    std::vector<double> wp(3 * (size_t)np), om(3 * (size_t)np);
    CK(cudaMemcpyAsync(wp.data(), ctx->wp, wp.size() * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaMemcpyAsync(om.data(), ctx->omgp, om.size() * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < 3; ++c) {
      part_mean_rms(wp, np, c, &wmn[c], &wrms[c]);
      part_mean_rms(om, np, c, &omn[c], &orms[c]);
    }
  }
  auto norm = [](double a, double b, double c) { return std::sqrt(a * a + b * b + c * c); };
  const double velfrms = norm(fl[4], fl[5], fl[6]);
  const double omgfrms = norm(fl[10], fl[11], fl[12]);
  double o[36] = {nf, nf / nx3,
                  fl[1], fl[2], fl[3], fl[4], fl[5], fl[6], velfrms, norm(fl[1], fl[2], fl[3]),
                  wmn[0], wmn[1], wmn[2], wrms[0], wrms[1], wrms[2], norm(wrms[0], wrms[1], wrms[2]),
                  norm(wmn[0], wmn[1], wmn[2]),
                  fl[7], fl[8], fl[9], fl[10], fl[11], fl[12], omgfrms / 2.0, norm(fl[7], fl[8], fl[9]),
                  omn[0], omn[1], omn[2], orms[0], orms[1], orms[2], norm(orms[0], orms[1], orms[2]),
                  // saveload.f90:1694 takes omgpxmn twice
                  norm(omn[0], omn[1], omn[0]),
                  omgfrms * omgfrms, velfrms * velfrms};
  std::memcpy(out, o, sizeof o);
  CK(cudaGetLastError());
  return LBM_OK;
}

int lbm_channel_profiles(lbm_ctx* ctx, int fluid_only, double ustar, double* out) {
  if (!ctx || !out) return LBM_ERR_ARG;
  if (int rc = poll_status(ctx)) return rc;
  if (!(ustar > 0.0)) {
    // force_in_y = 2 rho0 ustar^2 / nx (C/para.f90:15-17)
    const double fy = ctx->cfg.force_y;
    if (!(fy > 0.0)) return fail(ctx, LBM_ERR_ARG, "profiles: ustar not given and no channel force");
    ustar = std::sqrt(fy * ctx->g.nx / (2.0 * ctx->cfg.rho0));
  }
  materialize_macro(ctx);
  const int nx = ctx->g.nx;
  std::vector<double> sm((size_t)nx * 12);
  int rc = ctx->f32 ? plane_sums<float>(ctx->g, ctx->flags[ctx->fcur], fluid_only ? 1 : 0,
                                        mbuf<float>(ctx, 0), mbuf<float>(ctx, 1), mbuf<float>(ctx, 2),
                                        mbuf<float>(ctx, 3), sm.data(), ctx->stream)
                    : plane_sums<double>(ctx->g, ctx->flags[ctx->fcur], fluid_only ? 1 : 0,
                                         mbuf<double>(ctx, 0), mbuf<double>(ctx, 1),
                                         mbuf<double>(ctx, 2), mbuf<double>(ctx, 3), sm.data(),
                                         ctx->stream);
  if (rc) {
    cudaGetLastError();
    return fail(ctx, rc, "profiles: reduction failed");
  }
  const double ystar = ctx->cfg.visc / ustar;  // C/para.f90:18
  const int lxh = nx / 2;
  const double nyz = (double)ctx->g.ny * ctx->g.nz;
  const int ncol = fluid_only ? 15 : 13;
  for (int i = 1; i <= nx; ++i) {
    const double* a = &sm[(size_t)(i - 1) * 12];
    // statistc divides by ny*nz, statistc2 by the plane's fluid count
    const double cnt = fluid_only ? a[11] : nyz;
    const double u = a[0] / cnt / ustar, v = a[1] / cnt / ustar, w = a[2] / cnt / ustar;
    const double us2 = ustar * ustar;
    double* o = out + (size_t)(i - 1) * ncol;
    o[0] = (double)i - 0.5;
    o[1] = i > lxh ? ((double)(nx - i) + 0.5) / ystar : ((double)i - 0.5) / ystar;
    o[2] = u; o[3] = v; o[4] = w;
    o[5] = a[6] / cnt / us2 - u * u;
    o[6] = a[7] / cnt / us2 - v * v;
    o[7] = a[8] / cnt / us2 - w * w;
    o[8] = a[3] / cnt / us2 - u * w;
    o[9] = a[4] / cnt / us2 - u * v;
    o[10] = a[5] / cnt / us2 - v * w;
    const double pm = a[9] / cnt / us2;
    o[11] = pm;
    o[12] = a[10] / cnt / (us2 * us2) - pm * pm;
    if (fluid_only) {
      o[13] = a[11] / nyz;
      o[14] = 1.0 - o[13];
    }
  }
  return LBM_OK;
}

int lbm_diag(lbm_ctx* ctx, double* out) {
  if (!ctx || !out) return LBM_ERR_ARG;
  if (int rc = poll_status(ctx)) return rc;
  materialize_macro(ctx);
  double vmax = 0.0;
  int rc = ctx->f32 ? fluid_vmax<float>(ctx->g, ctx->flags[ctx->fcur], mbuf<float>(ctx, 1),
                                        mbuf<float>(ctx, 2), mbuf<float>(ctx, 3), &ctx->spec,
                                        &vmax, ctx->stream)
                    : fluid_vmax<double>(ctx->g, ctx->flags[ctx->fcur], mbuf<double>(ctx, 1),
                                         mbuf<double>(ctx, 2), mbuf<double>(ctx, 3), &ctx->spec,
                                         &vmax, ctx->stream);
  if (rc) {
    cudaGetLastError();
    return fail(ctx, rc, "diag: reduction failed");
  }
  double o[5] = {vmax, 0.0, 0.0, 0.0, 0.0};
  const int np = ctx->particles_on ? ctx->npart : 0;
  if (np > 0) {
    std::vector<double> wp(3 * (size_t)np), om(3 * (size_t)np);
    CK(cudaMemcpyAsync(wp.data(), ctx->wp, wp.size() * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaMemcpyAsync(om.data(), ctx->omgp, om.size() * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    // maxval and the first maxloc (1-based) of the magnitudes
    for (int which = 0; which < 2; ++which) {
      const std::vector<double>& v = which ? om : wp;
      double best = -1.0;
      int at = 0;
      for (int p = 0; p < np; ++p) {
        const double m = std::sqrt(v[3 * p] * v[3 * p] + v[3 * p + 1] * v[3 * p + 1] +
                                   v[3 * p + 2] * v[3 * p + 2]);
        if (m > best) { best = m; at = p + 1; }
      }
      o[1 + 2 * which] = at;
      o[2 + 2 * which] = best;
    }
  }
  std::memcpy(out, o, sizeof o);
  return LBM_OK;
}

int lbm_particle_slip(lbm_ctx* ctx, double r_in, double r_out, double* slip) {
  if (!ctx || !slip || !(r_out > r_in) || r_in < 0.0) return LBM_ERR_ARG;
  if (ctx->npart <= 0) return LBM_OK;
  if (int rc = poll_status(ctx)) return rc;
  materialize_macro(ctx);
  double* d = nullptr;
  CK(cudaMalloc((void**)&d, 3 * (size_t)ctx->npart * sizeof(double)));
  if (ctx->f32)
    launch_slip<float>(ctx->g, pview(ctx), mbuf<float>(ctx, 1), mbuf<float>(ctx, 2),
                       mbuf<float>(ctx, 3), ctx->flags[ctx->fcur], r_in, r_out, d, ctx->stream);
  else
    launch_slip<double>(ctx->g, pview(ctx), mbuf<double>(ctx, 1), mbuf<double>(ctx, 2),
                        mbuf<double>(ctx, 3), ctx->flags[ctx->fcur], r_in, r_out, d, ctx->stream);
  cudaError_t e = cudaMemcpyAsync(slip, d, 3 * (size_t)ctx->npart * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  CK(e);
  return LBM_OK;
}

int lbm_download_force(lbm_ctx* ctx, double* fx, double* fy, double* fz) {
  if (!ctx || !fx || !fy || !fz) return LBM_ERR_ARG;
  const long long N = ctx->g.N;
  double* d = nullptr;
  CK(cudaMalloc((void**)&d, 3 * N * sizeof(double)));
  if (ctx->f32)
    launch_force_field<float>(ctx->g, fview<float>(ctx, ctx->latest), d, d + N, d + 2 * N, ctx->stream);
  else
    launch_force_field<double>(ctx->g, fview<double>(ctx, ctx->latest), d, d + N, d + 2 * N, ctx->stream);
  cudaMemcpyAsync(fx, d, N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaMemcpyAsync(fy, d + N, N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaMemcpyAsync(fz, d + 2 * N, N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  if (e != cudaSuccess) return fail(ctx, LBM_ERR_CUDA, cudaGetErrorString(e));
  return LBM_OK;
}

int lbm_upload_particles(lbm_ctx* ctx, int npart, const double* ypglb, const double* wp,
                         const double* omgp) {
  if (!ctx || npart < 0 || npart > ctx->npmax) return LBM_ERR_ARG;
  if (npart > 0 && (!ypglb || !wp || !omgp)) return LBM_ERR_ARG;
  materialize_macro(ctx);
  size_t v = 3 * (size_t)ctx->npmax;
  if (ctx->npmax > 0) CK(cudaMemsetAsync(ctx->pbuf, 0, 15 * v * sizeof(double), ctx->stream));
  ctx->npart = npart;
  if (npart > 0) {
    size_t b = 3 * (size_t)npart * sizeof(double);
    CK(cudaMemcpyAsync(ctx->ypglb, ypglb, b, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->ypglbp, ypglb, b, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->wp, wp, b, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->omgp, omgp, b, cudaMemcpyHostToDevice, ctx->stream));
    int one = 1;
    CK(cudaMemcpyAsync(ctx->first_move, &one, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  }
  CK(reset_flags(ctx, 0));
  CK(reset_flags(ctx, 1));
  ctx->particles_on = npart > 0;
  if (npart > 0) launch_links(ctx->g, pview(ctx), ctx->flags[ctx->fcur], ctx->links, ctx->status, ctx->f32 ? 1 : 0, ctx->stream);
  CK(cudaGetLastError());
  return check_status(ctx);
}

int lbm_initpartvel(lbm_ctx* ctx, int npart, const double* ypglb, double* wp) {
  if (!ctx || npart < 0 || (npart > 0 && (!ypglb || !wp))) return LBM_ERR_ARG;
  if (npart == 0) return LBM_OK;
  materialize_macro(ctx);
  const size_t b = 3 * (size_t)npart * sizeof(double);
  char* scratch = nullptr;
  CK(cudaMallocAsync(reinterpret_cast<void**>(&scratch), 2 * b + 16, ctx->stream));
  double* dy = reinterpret_cast<double*>(scratch);
  double* dw = reinterpret_cast<double*>(scratch + b);
  int* dbad = reinterpret_cast<int*>(scratch + 2 * b);
  int bad = npart;
  CK(cudaMemcpyAsync(dy, ypglb, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(dbad, &bad, sizeof bad, cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->f32)
    launch_initpartvel<float>(ctx->g, mbuf<float>(ctx, 1), mbuf<float>(ctx, 2), mbuf<float>(ctx, 3),
                              dy, npart, dw, dbad, ctx->stream);
  else
    launch_initpartvel<double>(ctx->g, mbuf<double>(ctx, 1), mbuf<double>(ctx, 2),
                               mbuf<double>(ctx, 3), dy, npart, dw, dbad, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(wp, dw, b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&bad, dbad, sizeof bad, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaFreeAsync(scratch, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (bad < npart) return fail(ctx, LBM_ERR_ARG, "initpartvel: a centre's cell leaves the grid");
  return LBM_OK;
}

int lbm_release_particles(lbm_ctx* ctx, int npart, const double* ypglb) {
  if (!ctx || npart < 0 || npart > ctx->npmax || (npart > 0 && !ypglb)) return LBM_ERR_ARG;
  std::vector<double> wp(3 * (size_t)npart), omgp(3 * (size_t)npart, 0.0);
  if (int rc = lbm_initpartvel(ctx, npart, ypglb, wp.data())) return rc;
  return lbm_upload_particles(ctx, npart, ypglb, wp.data(), omgp.data());
}

int lbm_particle_state(lbm_ctx* ctx, int dir, int npart, double* state, int32_t* first_move) {
  if (!ctx || (dir != 0 && dir != 1) || npart < 0 || (npart > 0 && !state)) return LBM_ERR_ARG;
  if (ctx->in_batch && dir != 0)
    return fail(ctx, LBM_ERR_STATE, "the particle state of a batched context is read-only");
  double* vecs[15] = {ctx->ypglb, ctx->ypglbp, ctx->wp, ctx->wpp, ctx->omgp,
                      ctx->omgpp, ctx->dwdt, ctx->domgdt, ctx->forcep, ctx->forcepp,
                      ctx->torqp, ctx->torqpp, ctx->thetap, ctx->fHIp, ctx->flubp};
  const size_t b = 3 * (size_t)npart * sizeof(double);
  if (dir == 0) {
    if (npart != ctx->npart) return fail(ctx, LBM_ERR_ARG, "npart differs from the context's");
    for (int i = 0; i < 15 && npart > 0; ++i)
      CK(cudaMemcpyAsync(state + (size_t)i * 3 * npart, vecs[i], b, cudaMemcpyDeviceToHost,
                         ctx->stream));
    int fm = 0;
    if (ctx->first_move)
      CK(cudaMemcpyAsync(&fm, ctx->first_move, sizeof fm, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (first_move) *first_move = fm;
    return LBM_OK;
  }
  if (npart > ctx->npmax) return fail(ctx, LBM_ERR_ARG, "npart above the context's capacity");
  materialize_macro(ctx);
  if (ctx->npmax > 0)
    CK(cudaMemsetAsync(ctx->pbuf, 0, 15 * 3 * (size_t)ctx->npmax * sizeof(double), ctx->stream));
  for (int i = 0; i < 15 && npart > 0; ++i)
    CK(cudaMemcpyAsync(vecs[i], state + (size_t)i * 3 * npart, b, cudaMemcpyHostToDevice,
                       ctx->stream));
  if (ctx->first_move) {
    const int fm = first_move ? *first_move : 0;
    CK(cudaMemcpyAsync(ctx->first_move, &fm, sizeof fm, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));  // fm lives on this stack frame
  }
  ctx->npart = npart;
  CK(reset_flags(ctx, 0));
  CK(reset_flags(ctx, 1));
  ctx->particles_on = npart > 0;
  if (npart > 0)
    launch_links(ctx->g, pview(ctx), ctx->flags[ctx->fcur], ctx->links, ctx->status, ctx->f32 ? 1 : 0,
                 ctx->stream);
  CK(cudaGetLastError());
  return check_status(ctx);
}

int lbm_download_particles(lbm_ctx* ctx, double* ypglb, double* wp, double* omgp, double* fHIp,
                           double* flubp, double* torqp) {
  if (!ctx) return LBM_ERR_ARG;
  size_t b = 3 * (size_t)ctx->npart * sizeof(double);
  if (b == 0) return LBM_OK;
  double* outs[6] = {ypglb, wp, omgp, fHIp, flubp, torqp};
  double* srcs[6] = {ctx->ypglb, ctx->wp, ctx->omgp, ctx->fHIp, ctx->flubp, ctx->torqp};
  for (int i = 0; i < 6; ++i)
    if (outs[i]) CK(cudaMemcpyAsync(outs[i], srcs[i], b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return LBM_OK;
}

int lbm_download_flags(lbm_ctx* ctx, int32_t* ibnodes, int32_t* isnodes) {
  if (!ctx) return LBM_ERR_ARG;
  const long long N = ctx->g.N;
  std::vector<int32_t> tmp;
  int32_t* dst = isnodes;
  if (!dst) { tmp.resize(N); dst = tmp.data(); }
  CK(cudaMemcpyAsync(dst, ctx->flags[ctx->fcur], N * sizeof(int32_t), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (ibnodes)
    for (long long n = 0; n < N; ++n) ibnodes[n] = dst[n] >= 0 ? 1 : -1;
  return LBM_OK;
}

int lbm_download_links(lbm_ctx* ctx, int64_t capacity, int64_t* nlinks, int32_t* node,
                       int32_t* ipop, int32_t* particle, double* alpha) {
  if (!ctx || !nlinks) return LBM_ERR_ARG;
  *nlinks = 0;
  if (ctx->npart <= 0) return LBM_OK;
  std::vector<int32_t> cnt(ctx->npart);
  CK(cudaMemcpyAsync(cnt.data(), ctx->links.count, ctx->npart * sizeof(int32_t),
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  int64_t total = 0;
  for (int p = 0; p < ctx->npart; ++p) total += cnt[p];
  *nlinks = total;
  if (!node && !ipop && !particle && !alpha) return LBM_OK;
  if (capacity < total) return fail(ctx, LBM_ERR_CAPACITY, "link buffer too small");
  const int cap = ctx->links.cap;
  std::vector<int32_t> code((size_t)ctx->npart * cap);
  std::vector<double> al((size_t)ctx->npart * cap);
  CK(cudaMemcpyAsync(code.data(), ctx->links.code, code.size() * sizeof(int32_t),
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(al.data(), ctx->links.alpha, al.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  int64_t w = 0;
  for (int p = 0; p < ctx->npart; ++p)
    for (int l = 0; l < cnt[p]; ++l, ++w) {
      int32_t cd = code[(size_t)p * cap + l];
      if (node) node[w] = cd >> 5;
      if (ipop) ipop[w] = cd & 31;
      if (particle) particle[w] = p;
      if (alpha)
        alpha[w] = ctx->f32 ? (double)reinterpret_cast<const float*>(&al[(size_t)p * cap])[l]
                            : al[(size_t)p * cap + l];
    }
  return LBM_OK;
}

int lbm_forcing_state(lbm_ctx* ctx, int dir, int32_t* iseedf, int32_t* iyf, int32_t* ivf,
                      double* b) {
  if (!ctx) return LBM_ERR_ARG;
  if (ctx->in_batch && dir != 0)
    return fail(ctx, LBM_ERR_STATE, "the forcing state of a batched context is read-only");
  cancel_prefetch(ctx);
  if (ctx->cfg.forcing != LBM_FORCING_STOCHASTIC) return fail(ctx, LBM_ERR_STATE, "no stochastic forcing");
  ForcingDev st;
  if (ctx->side) CK(cudaStreamSynchronize(ctx->side));
  // in a batch the next step's FORCING may have run ahead: report the state
  // after the last completed step
  CK(cudaMemcpyAsync(&st, ctx->batch_ready ? ctx->d_forcing_backup : ctx->d_forcing, sizeof st,
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (dir == 0) {
    if (iseedf) *iseedf = st.iseedf;
    if (iyf) *iyf = st.iyf;
    if (ivf) std::memcpy(ivf, st.ivf, sizeof st.ivf);
    if (b) std::memcpy(b, st.b, sizeof st.b);
  } else {
    if (iseedf) st.iseedf = *iseedf;
    if (iyf) st.iyf = *iyf;
    if (ivf) std::memcpy(st.ivf, ivf, sizeof st.ivf);
    if (b) std::memcpy(st.b, b, sizeof st.b);
    CK(cudaMemcpyAsync(ctx->d_forcing, &st, sizeof st, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return LBM_OK;
}

// ---- per-subroutine entries ----------------------------------------------
int lbm_forcing(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  materialize_macro(ctx);
  do_forcing(ctx);
  CK(cudaGetLastError());
  return LBM_OK;
}

int lbm_collision_mrt(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  materialize_macro(ctx);
  if (ctx->f32)
    launch_collision<float>(ctx->g, ctx->r, fbuf<float>(ctx, ctx->cur), ctx->flags[ctx->fcur],
                            fview<float>(ctx, ctx->latest), mbuf<float>(ctx, 0), mbuf<float>(ctx, 1),
                            mbuf<float>(ctx, 2), mbuf<float>(ctx, 3), ctx->stream);
  else
    launch_collision<double>(ctx->g, ctx->r, fbuf<double>(ctx, ctx->cur), ctx->flags[ctx->fcur],
                             fview<double>(ctx, ctx->latest), mbuf<double>(ctx, 0),
                             mbuf<double>(ctx, 1), mbuf<double>(ctx, 2), mbuf<double>(ctx, 3),
                             ctx->stream);
  ctx->macro_derived = false;
  CK(cudaGetLastError());
  return LBM_OK;
}

int lbm_beads_collision(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  if (!ctx->particles_on) return LBM_OK;
  materialize_macro(ctx);
  if (ctx->f32) {
    launch_bounce_back<float>(ctx->g, pview(ctx), fbuf<float>(ctx, ctx->cur), 0, ctx->flags[ctx->fcur],
                              ctx->links, ctx->fHIp, ctx->torqp, ctx->stream);
    launch_bounce_scatter<float>(ctx->g, pview(ctx), fbuf<float>(ctx, ctx->cur), 0, ctx->links, ctx->stream);
  } else {
    launch_bounce_back<double>(ctx->g, pview(ctx), fbuf<double>(ctx, ctx->cur), 0, ctx->flags[ctx->fcur],
                               ctx->links, ctx->fHIp, ctx->torqp, ctx->stream);
    launch_bounce_scatter<double>(ctx->g, pview(ctx), fbuf<double>(ctx, ctx->cur), 0, ctx->links, ctx->stream);
  }
  ctx->macro_derived = false;
  CK(cudaGetLastError());
  return LBM_OK;
}

int lbm_streaming(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  materialize_macro(ctx);
  if (ctx->f32)
    launch_streaming<float>(ctx->g, fbuf<float>(ctx, ctx->cur), fbuf<float>(ctx, 1 - ctx->cur), ctx->stream);
  else
    launch_streaming<double>(ctx->g, fbuf<double>(ctx, ctx->cur), fbuf<double>(ctx, 1 - ctx->cur), ctx->stream);
  ctx->cur = 1 - ctx->cur;
  ctx->macro_derived = false;
  CK(cudaGetLastError());
  return LBM_OK;
}

int lbm_beads_lubforce(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  if (!ctx->particles_on) return LBM_OK;
  launch_lubforce(ctx->g, ctx->npart, ctx->pp, mstate(ctx), ctx->stream);
  CK(cudaGetLastError());
  return LBM_OK;
}

int lbm_beads_move(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  if (!ctx->particles_on) return LBM_OK;
  launch_move(ctx->g, ctx->npart, ctx->pp, mstate(ctx), ctx->stream);
  CK(cudaGetLastError());
  return LBM_OK;
}

int lbm_beads_redistribute(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  if (!ctx->particles_on) return LBM_OK;
  launch_redistribute(ctx->g, ctx->npart, ctx->pp, mstate(ctx), ctx->status, ctx->stream);
  CK(cudaGetLastError());
  return check_status(ctx);
}

int lbm_beads_links(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  if (!ctx->particles_on) return LBM_OK;
  int nf = 1 - ctx->fcur;
  CK(reset_flags(ctx, nf));
  launch_links(ctx->g, pview(ctx), ctx->flags[nf], ctx->links, ctx->status, ctx->f32 ? 1 : 0, ctx->stream);
  ctx->fcur = nf;
  CK(cudaGetLastError());
  return check_status(ctx);
}

int lbm_beads_filling(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  if (!ctx->particles_on) return LBM_OK;
  materialize_macro(ctx);
  if (ctx->f32)
    launch_filling<float>(ctx->g, pview(ctx), ctx->pp, ctx->ypglbp, ctx->wpp, ctx->omgpp,
                          ctx->flags[ctx->fcur], ctx->flags[1 - ctx->fcur],
                          fbuf<float>(ctx, ctx->cur), ctx->fill, ctx->status, ctx->stream);
  else
    launch_filling<double>(ctx->g, pview(ctx), ctx->pp, ctx->ypglbp, ctx->wpp, ctx->omgpp,
                           ctx->flags[ctx->fcur], ctx->flags[1 - ctx->fcur],
                           fbuf<double>(ctx, ctx->cur), ctx->fill, ctx->status, ctx->stream);
  ctx->macro_derived = false;
  CK(cudaGetLastError());
  return LBM_OK;
}

int lbm_macrovar(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  ctx->fmacro = ctx->latest;
  ctx->macro_pending = true;
  materialize_macro(ctx);
  CK(cudaGetLastError());
  return LBM_OK;
}

int lbm_rhoupdat(lbm_ctx* ctx) {
  if (!ctx) return LBM_ERR_ARG;
  materialize_macro(ctx);
  if (ctx->f32)
    launch_rhoupdat<float>(ctx->g, fbuf<float>(ctx, ctx->cur), mbuf<float>(ctx, 0), ctx->stream);
  else
    launch_rhoupdat<double>(ctx->g, fbuf<double>(ctx, ctx->cur), mbuf<double>(ctx, 0), ctx->stream);
  ctx->macro_derived = false;
  CK(cudaGetLastError());
  return LBM_OK;
}

int lbm_prerelax(lbm_ctx* ctx, double eps, int max_iter, int* iters, double* err) {
  if (!ctx || !(eps >= 0.0) || max_iter < 0) return LBM_ERR_ARG;
  if (ctx->in_batch) return fail(ctx, LBM_ERR_STATE, "a batched context steps only through its batch");
  materialize_macro(ctx);
  unsigned long long* maxbits = reinterpret_cast<unsigned long long*>(ctx->partial);
  int istep = 0;
  double e = 0.0;
  for (;;) {
    if (int rc = lbm_collision_mrt(ctx)) return rc;
    if (int rc = lbm_streaming(ctx)) return rc;
    if (ctx->f32)
      launch_rhoupdat_maxdiff<float>(ctx->g, fbuf<float>(ctx, ctx->cur), mbuf<float>(ctx, 0),
                                     maxbits, ctx->stream);
    else
      launch_rhoupdat_maxdiff<double>(ctx->g, fbuf<double>(ctx, ctx->cur), mbuf<double>(ctx, 0),
                                      maxbits, ctx->stream);
    unsigned long long bits = 0;
    CK(cudaMemcpyAsync(&bits, maxbits, sizeof bits, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    std::memcpy(&e, &bits, sizeof e);
    if (!std::isfinite(e)) return fail(ctx, LBM_ERR_NONFINITE, "pre-relaxation: density not finite");
    if (e <= eps || istep > max_iter) break;
    ++istep;
  }
  ctx->macro_derived = false;
  if (iters) *iters = istep;
  if (err) *err = e;
  return LBM_OK;
}

// Report a device error raised by an earlier lbm_step without blocking:
// the status word is copied back asynchronously at the end of each call.
static int poll_status(lbm_ctx* ctx) {
  if (!ctx->status_pending) return 0;
  if (cudaEventQuery(ctx->ev_status) != cudaSuccess) return 0;
  ctx->status_pending = false;
  if (ctx->status_host->code == 0) return 0;
  return check_status(ctx);
}

int lbm_step(lbm_ctx* ctx, int nsteps) {
  if (!ctx || nsteps < 0) return LBM_ERR_ARG;
  if (ctx->in_batch) return fail(ctx, LBM_ERR_STATE, "the context is stepped by its batch");
  if (int rc = poll_status(ctx)) return rc;
  for (int s = 0; s < nsteps; ++s) {
    if (!ctx->macro_derived) {
      if (ctx->f32) unfused_step_t<float>(ctx); else unfused_step_t<double>(ctx);
    } else {
      if (ctx->f32) fused_step_t<float>(ctx); else fused_step_t<double>(ctx);
    }
  }
  CK(cudaGetLastError());
  if (ctx->particles_on || ctx->variant != LBM_VARIANT_DIRECT) {
    CK(cudaMemcpyAsync(ctx->status_host, ctx->status, sizeof(DevStatus), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaEventRecord(ctx->ev_status, ctx->stream));
    ctx->status_pending = true;
  }
  return LBM_OK;
}

int lbm_set_variant(lbm_ctx* ctx, int variant, int stages, int groups, int ctas_per_sm) {
  if (!ctx) return LBM_ERR_ARG;
  if (variant == LBM_VARIANT_DIRECT) {
    ctx->variant = variant;
    return LBM_OK;
  }
  if ((variant != LBM_VARIANT_STAGED && variant != LBM_VARIANT_STAGED_X2) || stages < 0 ||
      stages > 8 || groups < 0 || groups > 8 || ctas_per_sm < 0)
    return fail(ctx, LBM_ERR_ARG, "unknown stream+collide variant or schedule");
  StagedPlan p;
  if (!plan_staged(ctx, variant, stages, ctas_per_sm, &p, groups == 0 ? 1 : groups)) {
    cudaGetLastError();
    return fail(ctx, LBM_ERR_ARG, "this stream+collide variant does not apply to this box");
  }
  ctx->variant = variant;
  ctx->staged = p;
  return LBM_OK;
}

int lbm_set_sums(lbm_ctx* ctx, int mode) {
  if (!ctx) return LBM_ERR_ARG;
  if (mode != LBM_SUMS_FLOAT && mode != LBM_SUMS_FIXED && mode != LBM_SUMS_INTEGER)
    return fail(ctx, LBM_ERR_ARG, "unknown collision arithmetic");
  if (ctx->f32 && mode != LBM_SUMS_FLOAT)
    return fail(ctx, LBM_ERR_ARG, "fixed-point sums apply to FP64 contexts only");
  const int keep = ctx->sums;
  ctx->sums = mode;
  if (ctx->variant != LBM_VARIANT_DIRECT) {
    // the staged kernel differs: re-plan the same schedule for it
    StagedPlan p;
    if (!plan_staged(ctx, ctx->variant, ctx->staged.S, ctx->staged.ctas_per_sm, &p,
                     ctx->staged.groups)) {
      cudaGetLastError();
      ctx->sums = keep;
      return fail(ctx, LBM_ERR_ARG, "the current stream+collide schedule does not apply");
    }
    ctx->staged = p;
  }
  return LBM_OK;
}

int lbm_get_sums(lbm_ctx* ctx, int* mode) {
  if (!ctx || !mode) return LBM_ERR_ARG;
  *mode = ctx->sums;
  return LBM_OK;
}

int lbm_get_variant(lbm_ctx* ctx, int* variant, int* stages, int* groups, int* ctas_per_sm) {
  if (!ctx) return LBM_ERR_ARG;
  if (variant) *variant = ctx->variant;
  const bool st = ctx->variant != LBM_VARIANT_DIRECT;
  if (stages) *stages = st ? ctx->staged.S : 0;
  if (groups) *groups = st ? ctx->staged.groups : 0;
  if (ctas_per_sm) *ctas_per_sm = st ? ctx->staged.ctas_per_sm : 0;
  return LBM_OK;
}

int lbm_autotune(lbm_ctx* ctx, int reps, double* best_ms) {
  if (!ctx || reps < 1) return LBM_ERR_ARG;
  if (int rc = poll_status(ctx)) return rc;
  struct Cand { int variant; StagedPlan p; };
  std::vector<Cand> cands;
  cands.push_back({LBM_VARIANT_DIRECT, StagedPlan{}});
  for (int variant : {LBM_VARIANT_STAGED, LBM_VARIANT_STAGED_X2})
    for (int groups = 1; groups <= 8; ++groups)
      for (int S = 2; S <= 8; ++S)
        for (int per_sm : {1, 2, 3, 4}) {
          StagedPlan p;
          if (!plan_staged(ctx, variant, S, per_sm, &p, groups)) continue;
          bool dup = false;
          for (const Cand& c : cands)
            dup |= c.variant == variant && c.p.S == p.S && c.p.ctas_per_sm == p.ctas_per_sm &&
                   c.p.groups == p.groups;
          if (!dup) cands.push_back({variant, p});
        }
  cudaGetLastError();
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int keep_variant = ctx->variant;
  const StagedPlan keep_plan = ctx->staged;
  double best = 1e30;
  size_t best_i = 0;
  const bool prof = ctx->prof_on;
  ctx->prof_on = false;
  for (size_t i = 0; i < cands.size(); ++i) {
    ctx->variant = cands[i].variant;
    ctx->staged = cands[i].p;
    // the direct FP64 candidate is timed on fixed-point populations, as its
    // fused steps run
    if (fixed_path(ctx)) pop_format(ctx, true);
    auto run = [&]() {
      if (ctx->f32) launch_stream_collide<float>(ctx, fbuf<float>(ctx, ctx->cur), fbuf<float>(ctx, 1 - ctx->cur));
      else if (ctx->g.pop_fixed)
        launch_stream_collide<double>(ctx, fraw<double>(ctx, ctx->cur), fraw<double>(ctx, 1 - ctx->cur));
      else launch_stream_collide<double>(ctx, fbuf<double>(ctx, ctx->cur), fbuf<double>(ctx, 1 - ctx->cur));
    };
    run();
    cudaEventRecord(e0, ctx->stream);
    for (int k = 0; k < reps; ++k) run();
    cudaEventRecord(e1, ctx->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms / reps < best) { best = ms / reps; best_i = i; }
  }
  ctx->prof_on = prof;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->variant = keep_variant;
  ctx->staged = keep_plan;
  CK(cudaGetLastError());
  if (int rc = check_status(ctx)) return rc;
  ctx->variant = cands[best_i].variant;
  ctx->staged = cands[best_i].p;
  if (best_ms) *best_ms = best;
  return LBM_OK;
}

int lbm_profile(lbm_ctx* ctx, int enable) {
  if (!ctx) return LBM_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->prof_on = enable != 0;
  if (enable) {
    ctx->ev_used = 0;
    ctx->intervals.clear();
  }
  return LBM_OK;
}

int lbm_profile_read(lbm_ctx* ctx, int phase, double* ms_total, int64_t* count) {
  if (!ctx || phase < 0 || phase >= LBM_NPHASES) return LBM_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  double tot = 0.0;
  int64_t n = 0;
  for (const auto& iv : ctx->intervals) {
    if (iv.phase != phase) continue;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev_pool[iv.e0], ctx->ev_pool[iv.e1]));
    tot += ms;
    ++n;
  }
  if (ms_total) *ms_total = tot;
  if (count) *count = n;
  return LBM_OK;
}

int64_t lbm_kernel_launches(void) { return g_launches.load(); }

int lbm_mass_momentum(lbm_ctx* ctx, double out[4]) {
  if (!ctx || !out) return LBM_ERR_ARG;
  const int nb = 1024;
  if (ctx->f32)
    launch_mass_momentum<float>(ctx->g, fbuf<float>(ctx, ctx->cur), ctx->partial, nb, ctx->stream);
  else
    launch_mass_momentum<double>(ctx->g, fbuf<double>(ctx, ctx->cur), ctx->partial, nb, ctx->stream);
  CK(cudaMemcpyAsync(ctx->partial_host, ctx->partial, 4 * nb * sizeof(double),
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int c = 0; c < 4; ++c) out[c] = 0.0;
  for (int b = 0; b < nb; ++b)
    for (int c = 0; c < 4; ++c) out[c] += ctx->partial_host[4 * b + c];
  return LBM_OK;
}


}  // extern "C"

// ---------------------------------------------------------------------------
// lbm_batch: many contexts advanced together
struct lbm_batch {
  std::vector<lbm_ctx*> ctx;
  cudaStream_t main = nullptr;
  bool own_main = false;
  bool channel = false;
  Rates r;
  BatchBox* d_boxes = nullptr;
  BatchTask* d_tasks = nullptr;
  int ntasks = 0;
  long long nodes = 0;
  StagedPlan plan;
  DevStatus* status = nullptr;
  cudaEvent_t ev_fork = nullptr;
  std::vector<cudaEvent_t> ev_join;
  cudaGraphExec_t graph = nullptr;
  int graph_key[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
  std::vector<cudaEvent_t> ev_side;
  // particle step and FORCING of all boxes, one launch per kernel
  BoxParticles* d_parts[2] = {nullptr, nullptr};  // per buffer parity
  BoxForcing* d_forcing = nullptr;
  int max_npart = 0, max_nz = 0;
  long long max_reset = 0, max_rows = 0;
  bool stochastic = false;
  cudaStream_t side = nullptr;
  cudaEvent_t ev_side_all = nullptr;
  int64_t graph_kernels = 0;
  std::string err;
};

namespace {

constexpr int kBatchCycle = 6;  // buffer parity (2) x forcing slot rotation (3)

int bfail(lbm_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  return code;
}
#define BK(call)                                                                     \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return bfail(b, LBM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

constexpr int kKey = 8;
void phase_key(const lbm_ctx* c, int k[kKey]) {
  k[0] = c->cur; k[1] = c->fcur;
  k[2] = c->latest.mode; k[3] = c->latest.slot;
  k[4] = c->fmacro.mode; k[5] = c->fmacro.slot;
  k[6] = c->batch_ready; k[7] = c->batch_slot;
}

bool same_phase(const lbm_batch* b) {
  int k0[kKey], k[kKey];
  phase_key(b->ctx[0], k0);
  for (lbm_ctx* c : b->ctx) {
    phase_key(c, k);
    for (int i = 0; i < kKey; ++i)
      if (k[i] != k0[i]) return false;
    if (!c->macro_derived || c->prefetched) return false;
  }
  return true;
}

// One step of every box: the box's FORCING (prefetched during the previous
// step, else run now) on its stream, one stream + collide kernel for all
// boxes on the batch stream, then per box the next step's FORCING on its
// side stream alongside bounce-back and the particle subroutines on its
// stream; everything joins back into the batch stream.
// returns "" or the first call that failed (capture included)
std::string batch_step_eager(lbm_batch* b) {
  if (!same_phase(b)) return "the boxes are not at the same step phase";
  auto chk = [&](cudaError_t e, const char* what, size_t i) -> std::string {
    if (e != cudaSuccess)
      return std::string(what) + " (box " + std::to_string(i) + "): " + cudaGetErrorString(e);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(b->main, &cs);
    if (cs == cudaStreamCaptureStatusInvalidated)
      return std::string("capture invalidated after ") + what + " (box " + std::to_string(i) + ")";
    return "";
  };
  std::string err;
  // this step's FORCING: run during the previous step (joined since), or
  // constant, or (first step of a batch) now on each box's stream
  bool any_pending = false;
  std::vector<char> pending(b->ctx.size(), 0);
  for (size_t i = 0; i < b->ctx.size(); ++i) {
    lbm_ctx* c = b->ctx[i];
    if (c->batch_ready) {
      c->latest = {FM_TABLE, c->batch_slot};
      c->batch_ready = false;
    } else if (c->cfg.forcing == LBM_FORCING_STOCHASTIC) {
      pending[i] = 1;
      any_pending = true;
    } else {
      do_forcing(c);  // constant or none: no launch
    }
  }
  if (any_pending &&
      !(err = chk(cudaEventRecord(b->ev_fork, b->main), "fork", 0)).empty())
    return err;
  for (size_t i = 0; i < b->ctx.size() && any_pending; ++i) {
    lbm_ctx* c = b->ctx[i];
    if (!pending[i]) continue;
    if (!(err = chk(cudaStreamWaitEvent(c->stream, b->ev_fork, 0), "box wait", i)).empty()) return err;
    do_forcing(c);
    if (!(err = chk(cudaGetLastError(), "forcing", i)).empty()) return err;
    if (!(err = chk(cudaEventRecord(b->ev_join[i], c->stream), "join record", i)).empty()) return err;
    if (!(err = chk(cudaStreamWaitEvent(b->main, b->ev_join[i], 0), "join wait", i)).empty()) return err;
  }
  const lbm_ctx* c0 = b->ctx[0];
  BatchPhase ph{c0->cur, c0->fcur, c0->fmacro.mode, c0->fmacro.slot, c0->latest.mode,
                c0->latest.slot};
  launch_fused_batch(b->channel, b->d_boxes, b->d_tasks, b->ntasks, ph, b->r, b->plan, b->status,
                     b->main);
  if (!(err = chk(cudaGetLastError(), "batch kernel", 0)).empty()) return err;
  if (!(err = chk(cudaEventRecord(b->ev_fork, b->main), "fork 2", 0)).empty()) return err;
  const int par = c0->cur;  // buffer parity of this step (every box: cur == fcur)
  if (b->stochastic) {
    // the next step's FORCING of every box, one launch per kernel, on the
    // batch's side stream beside the particle step
    int slot = 0;
    for (int q = 0; q < 3; ++q)
      if (q != c0->latest.slot) { slot = q; break; }
    if (!(err = chk(cudaStreamWaitEvent(b->side, b->ev_fork, 0), "side wait", 0)).empty()) return err;
    launch_forcing_multi(b->d_forcing, (int)b->ctx.size(), b->max_nz, b->max_rows, slot, b->side);
    if (!(err = chk(cudaGetLastError(), "forcing", 0)).empty()) return err;
    if (!(err = chk(cudaEventRecord(b->ev_side_all, b->side), "side record", 0)).empty()) return err;
    for (lbm_ctx* c : b->ctx) {
      c->batch_ready = true;
      c->batch_slot = slot;
    }
  }
  launch_particle_step_multi(b->d_parts[par], (int)b->ctx.size(), b->max_npart, b->max_reset,
                             b->main);
  if (!(err = chk(cudaGetLastError(), "particles", 0)).empty()) return err;
  if (b->stochastic &&
      !(err = chk(cudaStreamWaitEvent(b->main, b->ev_side_all, 0), "side join", 0)).empty())
    return err;
  for (lbm_ctx* c : b->ctx) {  // host side of the step, as the end of fused_step_t
    c->fcur = 1 - c->fcur;
    c->cur = 1 - c->cur;
    c->fmacro = c->latest;
    c->macro_pending = true;
    c->macro_derived = true;
  }
  return "";
}

}  // namespace

extern "C" {

int lbm_batch_create(lbm_ctx** ctxs, int n, lbm_batch** out) {
  if (!ctxs || n < 1 || !out) return LBM_ERR_ARG;
  *out = nullptr;
  lbm_ctx* c0 = ctxs[0];
  if (!c0) return LBM_ERR_ARG;
  for (int i = 0; i < n; ++i) {
    lbm_ctx* c = ctxs[i];
    if (!c || !c->f32 || !batch_box_ok(c->g) || c->g.channel != c0->g.channel ||
        c->cfg.visc != c0->cfg.visc || c->cfg.mrt_type != c0->cfg.mrt_type ||
        c->cfg.forcing != c0->cfg.forcing || c->in_batch)
      return fail(c0, LBM_ERR_ARG,
                  "batch: every box must be FP32, nx a multiple of 4 and at most 128, with the "
                  "same boundary, viscosity, MRT rates and forcing, and in no other batch");
    for (int j = 0; j < i; ++j)
      if (ctxs[j] == c) return fail(c0, LBM_ERR_ARG, "batch: a context appears twice");
  }
  lbm_batch* b = new lbm_batch();
  b->ctx.assign(ctxs, ctxs + n);
  b->channel = c0->g.channel != 0;
  b->r = c0->r;
  for (lbm_ctx* c : b->ctx) {
    cancel_prefetch(c);
    cudaStreamSynchronize(c->stream);
    c->in_batch = true;
    c->fcache_slot = -1;
  }
  // boxes and tasks
  std::vector<BatchBox> boxes(n);
  std::vector<BatchTask> tasks;
  for (int i = 0; i < n; ++i) {
    lbm_ctx* c = b->ctx[i];
    BatchBox& x = boxes[i];
    x.nx = c->g.nx; x.ny = c->g.ny; x.nz = c->g.nz; x.sw = c->g.sw; x.N = (int)c->g.N;
    x.f[0] = static_cast<float*>(c->f[0]);
    x.f[1] = static_cast<float*>(c->f[1]);
    x.flags[0] = c->flags[0];
    x.flags[1] = c->flags[1];
    for (int s = 0; s < 3; ++s) x.rowtab[s] = static_cast<const float*>(c->rowtab[s]);
    x.xtw = static_cast<const float*>(c->xtw);
    x.cfx = 0.f; x.cfy = (float)c->cfg.force_y; x.cfz = 0.f;
    const int k = batch_task_rows(c->g.nx, c->g.ny);
    const int rows = c->g.ny * c->g.nz;
    for (int r0 = 0; r0 < rows; r0 += k) tasks.push_back({i, r0, k});
    b->nodes += c->g.N;
  }
  b->ntasks = (int)tasks.size();
  // per-box views of the particle step (both buffer parities) and FORCING
  std::vector<BoxParticles> parts(2 * (size_t)n);
  std::vector<BoxForcing> forc(n);
  b->stochastic = c0->cfg.forcing == LBM_FORCING_STOCHASTIC;
  for (int i = 0; i < n; ++i) {
    lbm_ctx* c = b->ctx[i];
    for (int par = 0; par < 2; ++par) {
      BoxParticles& x = parts[(size_t)par * n + i];
      x.g = c->g;
      x.pv = pview(c);
      if (!c->particles_on) x.pv.npart = 0;
      x.pp = c->pp;
      x.ms = mstate(c);
      x.ls = c->links;
      x.fl = c->fill;
      x.f = static_cast<float*>(c->f[1 - par]);
      x.flags_cur = c->flags[par];
      x.flags_next = c->flags[1 - par];
      x.st = c->status;
    }
    if (c->particles_on) {
      b->max_npart = std::max(b->max_npart, c->npart);
      b->max_reset = std::max(b->max_reset,
                              (long long)c->g.N + (long long)c->g.ny * c->g.nz * c->g.sw);
    }
    BoxForcing& fb = forc[i];
    fb.g = c->g;
    fb.st = c->d_forcing;
    fb.backup = c->d_forcing_backup;
    fb.var = c->var; fb.tf = c->tf; fb.pi2 = c->pi2;
    fb.kxr6 = c->d_kxr6; fb.kyr5 = c->d_kyr5; fb.kzr5 = c->d_kzr5;
    fb.ytw = static_cast<const float*>(c->ytw); fb.ztw = c->ztw;
    fb.ztab = static_cast<float*>(c->ztab);
    for (int q = 0; q < 3; ++q) fb.rowtab[q] = static_cast<float*>(c->rowtab[q]);
    b->max_nz = std::max(b->max_nz, c->g.nz);
    b->max_rows = std::max(b->max_rows, (long long)c->g.ny * c->g.nz);
  }
  int rc = 0;
  if (cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaMalloc((void**)&b->d_boxes, boxes.size() * sizeof(BatchBox)) != cudaSuccess ||
      cudaMalloc((void**)&b->d_tasks, tasks.size() * sizeof(BatchTask)) != cudaSuccess ||
      cudaMalloc((void**)&b->status, sizeof(DevStatus)) != cudaSuccess ||
      cudaMalloc((void**)&b->d_parts[0], parts.size() * sizeof(BoxParticles)) != cudaSuccess ||
      cudaMalloc((void**)&b->d_forcing, forc.size() * sizeof(BoxForcing)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_side_all, cudaEventDisableTiming) != cudaSuccess)
    rc = LBM_ERR_CUDA;
  if (!rc) b->d_parts[1] = b->d_parts[0] + n;
  b->own_main = true;
  b->ev_join.resize(n, nullptr);
  b->ev_side.resize(n, nullptr);
  for (int i = 0; i < n && !rc; ++i)
    if (cudaEventCreateWithFlags(&b->ev_join[i], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_side[i], cudaEventDisableTiming) != cudaSuccess)
      rc = LBM_ERR_CUDA;
  if (!rc) {
    cudaMemcpyAsync(b->d_boxes, boxes.data(), boxes.size() * sizeof(BatchBox),
                    cudaMemcpyHostToDevice, b->main);
    cudaMemcpyAsync(b->d_tasks, tasks.data(), tasks.size() * sizeof(BatchTask),
                    cudaMemcpyHostToDevice, b->main);
    cudaMemcpyAsync(b->d_parts[0], parts.data(), parts.size() * sizeof(BoxParticles),
                    cudaMemcpyHostToDevice, b->main);
    cudaMemcpyAsync(b->d_forcing, forc.data(), forc.size() * sizeof(BoxForcing),
                    cudaMemcpyHostToDevice, b->main);
    cudaMemsetAsync(b->status, 0, sizeof(DevStatus), b->main);
    if (!plan_batch(b->channel, 4, 2, 0, b->ntasks, &b->plan) &&
        !plan_batch(b->channel, 2, 1, 0, b->ntasks, &b->plan))
      rc = LBM_ERR_ARG;
  }
  if (!rc && cudaStreamSynchronize(b->main) != cudaSuccess) rc = LBM_ERR_CUDA;
  if (rc) {
    cudaGetLastError();
    lbm_batch_destroy(b);
    return rc;
  }
  *out = b;
  return LBM_OK;
}

int lbm_batch_destroy(lbm_batch* b) {
  if (!b) return LBM_OK;
  if (b->main) cudaStreamSynchronize(b->main);
  if (b->side) cudaStreamSynchronize(b->side);
  for (lbm_ctx* c : b->ctx) {
    if (c->side) cudaStreamSynchronize(c->side);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->batch_ready) {
      // the next step's FORCING ran ahead: restore the state before it
      cudaMemcpy(c->d_forcing, c->d_forcing_backup, sizeof(ForcingDev), cudaMemcpyDeviceToDevice);
      c->batch_ready = false;
    }
    c->in_batch = false;
    c->fcache_slot = -1;
  }
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (cudaEvent_t e : b->ev_join)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : b->ev_side)
    if (e) cudaEventDestroy(e);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  cudaFree(b->d_boxes);
  cudaFree(b->d_tasks);
  cudaFree(b->status);
  cudaFree(b->d_parts[0]);
  cudaFree(b->d_forcing);
  if (b->ev_side_all) cudaEventDestroy(b->ev_side_all);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->own_main && b->main) cudaStreamDestroy(b->main);
  delete b;
  return LBM_OK;
}

const char* lbm_batch_last_error(const lbm_batch* b) { return b ? b->err.c_str() : "no batch"; }

int lbm_batch_step(lbm_batch* b, int nsteps, int use_graph) {
  if (!b || nsteps < 0) return LBM_ERR_ARG;
  if (!same_phase(b))
    return bfail(b, LBM_ERR_STATE, "batch: the boxes are not at the same step phase");
  for (lbm_ctx* c : b->ctx) {
    if (c->prof_on) return bfail(b, LBM_ERR_STATE, "batch: profiling is on for a box");
  }
  BK(cudaGetLastError());  // nothing pending from earlier calls
  while (nsteps > 0) {
    if (use_graph && nsteps >= kBatchCycle) {
      int key[kKey];
      phase_key(b->ctx[0], key);
      bool match = b->graph != nullptr;
      for (int i = 0; i < kKey && match; ++i) match = key[i] == b->graph_key[i];
      if (!match) {
        if (b->graph) {
          cudaGraphExecDestroy(b->graph);
          b->graph = nullptr;
        }
        const int64_t l0 = g_launches.load();
        BK(cudaStreamBeginCapture(b->main, cudaStreamCaptureModeRelaxed));
        std::string err;
        for (int k = 0; k < kBatchCycle && err.empty(); ++k) err = batch_step_eager(b);
        cudaGraph_t gr = nullptr;
        cudaError_t ee = cudaStreamEndCapture(b->main, &gr);
        if (!err.empty() || ee != cudaSuccess) {
          if (gr) cudaGraphDestroy(gr);
          cudaGetLastError();
          return bfail(b, LBM_ERR_CUDA, "batch graph capture: " +
                                            (err.empty() ? std::string(cudaGetErrorString(ee)) : err));
        }
        cudaError_t e = cudaGraphInstantiate(&b->graph, gr, 0);
        cudaGraphDestroy(gr);
        BK(e);
        b->graph_kernels = g_launches.load() - l0;
        for (int i = 0; i < kKey; ++i) b->graph_key[i] = key[i];
        // capturing advanced the host state by one cycle; the replay below
        // performs that cycle on the device
        BK(cudaGraphLaunch(b->graph, b->main));
      } else {
        BK(cudaGraphLaunch(b->graph, b->main));
        g_launches.fetch_add(b->graph_kernels);
      }
      nsteps -= kBatchCycle;
    } else {
      const std::string err = batch_step_eager(b);
      if (!err.empty()) return bfail(b, LBM_ERR_CUDA, "batch step: " + err);
      --nsteps;
    }
  }
  BK(cudaGetLastError());
  return LBM_OK;
}

int lbm_batch_wait(lbm_batch* b) {
  if (!b) return LBM_ERR_ARG;
  BK(cudaStreamSynchronize(b->main));
  DevStatus st;
  BK(cudaMemcpy(&st, b->status, sizeof st, cudaMemcpyDeviceToHost));
  if (st.code) {
    cudaMemset(b->status, 0, sizeof(DevStatus));
    return bfail(b, st.code, "batch stream+collide kernel: a bounded wait ran out");
  }
  return LBM_OK;
}

int lbm_batch_synchronize(lbm_batch* b) {
  if (int rc = lbm_batch_wait(b)) return rc;
  for (lbm_ctx* c : b->ctx) {
    if (int rc = lbm_synchronize(c)) return bfail(b, rc, c->err);
  }
  return LBM_OK;
}

int lbm_batch_set_schedule(lbm_batch* b, int stages, int groups, int ctas_per_sm) {
  if (!b) return LBM_ERR_ARG;
  StagedPlan p;
  if (!plan_batch(b->channel, stages, groups, ctas_per_sm, b->ntasks, &p)) {
    cudaGetLastError();
    return bfail(b, LBM_ERR_ARG, "batch: schedule does not apply");
  }
  b->plan = p;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return LBM_OK;
}

int lbm_batch_get_schedule(lbm_batch* b, int* stages, int* groups, int* ctas_per_sm) {
  if (!b) return LBM_ERR_ARG;
  if (stages) *stages = b->plan.S;
  if (groups) *groups = b->plan.groups;
  if (ctas_per_sm) *ctas_per_sm = b->plan.ctas_per_sm;
  return LBM_OK;
}

int lbm_batch_autotune(lbm_batch* b, int reps, double* best_ms) {
  if (!b || reps < 1) return LBM_ERR_ARG;
  if (!same_phase(b)) return bfail(b, LBM_ERR_STATE, "batch: the boxes are not at the same step phase");
  BK(cudaDeviceSynchronize());
  const lbm_ctx* c0 = b->ctx[0];
  // the stream + collide of the current state (fin -> fout, nothing advances)
  BatchPhase ph{c0->cur, c0->fcur, c0->fmacro.mode, c0->fmacro.slot, c0->latest.mode,
                c0->latest.slot};
  cudaEvent_t e0, e1;
  BK(cudaEventCreate(&e0));
  BK(cudaEventCreate(&e1));
  const StagedPlan keep = b->plan;
  double best = 1e30;
  StagedPlan bestp = keep;
  for (int groups : {1, 2, 4})
    for (int S = 2; S <= 8; ++S)
      for (int per_sm : {1, 2, 3, 4, 6}) {
        StagedPlan p;
        if (!plan_batch(b->channel, S, groups, per_sm, b->ntasks, &p)) continue;
        if (p.ctas_per_sm != per_sm) continue;
        launch_fused_batch(b->channel, b->d_boxes, b->d_tasks, b->ntasks, ph, b->r, p, b->status,
                           b->main);
        cudaEventRecord(e0, b->main);
        for (int k = 0; k < reps; ++k)
          launch_fused_batch(b->channel, b->d_boxes, b->d_tasks, b->ntasks, ph, b->r, p,
                             b->status, b->main);
        cudaEventRecord(e1, b->main);
        if (cudaEventSynchronize(e1) != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms / reps < best) {
          best = ms / reps;
          bestp = p;
        }
      }
  cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->plan = best < 1e30 ? bestp : keep;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  if (int rc = lbm_batch_synchronize(b)) return rc;
  if (best_ms) *best_ms = best;
  return LBM_OK;
}

int64_t lbm_batch_nodes(const lbm_batch* b) { return b ? b->nodes : 0; }

int lbm_batch_set_stream(lbm_batch* b, void* stream) {
  if (!b) return LBM_ERR_ARG;
  BK(cudaStreamSynchronize(b->main));
  if (b->own_main) cudaStreamDestroy(b->main);
  if (stream) {
    b->main = static_cast<cudaStream_t>(stream);
    b->own_main = false;
  } else {
    BK(cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking));
    b->own_main = true;
  }
  return LBM_OK;
}

}  // extern "C"
