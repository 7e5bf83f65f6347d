// lbm_particles.cu - finite-size particle kernels (B/partlib.f90).
//
// Compiled with -fmad=false: the geometry that decides integer outcomes
// (solid flags, links, bounce-back branches, refill events) must round
// exactly like the CPU restatement, which evaluates the reference's
// expressions left to right without fused multiply-adds.
//
// Kernels (one block per particle unless noted):
//   k_links        beads_links   (B/partlib.f90:934-1058)  flags + link slabs
//   k_bounce       beads_collision (1363-1703)   interpolated bounce-back,
//                  momentum-exchange force/torque (deterministic block sums)
//   k_bounce_store the bounce-back stores, after every link has read
//   k_lubforce     beads_lubforce (2211-2292)   one thread per particle
//   k_move         beads_move (2295-2394)       one thread per particle
//   k_wrap / k_overlap  beads_redistribute's wrap and overlap check
//   k_filling      beads_filling (2793-3111)    refill of uncovered nodes
#include <cub/block/block_reduce.cuh>
#include <cub/block/block_scan.cuh>

#include "lbm_internal.cuh"
#include "lbm_collide.cuh"  // the fixed-point population format

namespace lbm {

namespace {

constexpr int PB = 256;  // threads per particle block
// One thread per particle (or per particle axis) with serial FP64 work: one
// warp per block spreads the particles over as many SMs as there are warps,
// since this GPU issues FP64 at a few lanes per clock per SM.
constexpr int kSmallBlock = 32;
constexpr int kBounceSpan = 64;  // coordinates per axis tabulated by beads_collision

__device__ __forceinline__ double near_img(double c, double p, int n, int nh) {
  if ((c - p) > (double)nh) c = c - (double)n;
  if ((c - p) < -(double)nh) c = c + (double)n;
  return c;
}
__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
// -v when neg, v otherwise, as a sign-bit flip: a negation that is not folded
// into an arithmetic operand would otherwise cost an FP64 add, and FP64
// issues at a few lanes per clock per SM on this GPU
__device__ __forceinline__ double flip_if(bool neg, double v) {
  return __longlong_as_double(
      (long long)((unsigned long long)__double_as_longlong(v) ^ ((unsigned long long)neg << 63)));
}
__device__ __forceinline__ float flip_if(bool neg, float v) {
  return __int_as_float((int)((unsigned)__float_as_int(v) ^ ((unsigned)neg << 31)));
}
template <typename R>
__device__ __forceinline__ R near_img_t(R c, R p, int n, int nh) {
  if ((c - p) > R(nh)) c = c - R(n);
  if ((c - p) < -R(nh)) c = c + R(n);
  return c;
}

// The reference's beads_links keeps shifting the particle centre toward the
// current point and never resets it inside its loop nest
// (B/partlib.f90:961-982): at point p_j = j - 0.5 of a sweep j = 1..n it
// applies "if (c - p > n/2) c -= n; if (c - p < -n/2) c += n" to the value
// left by the previous point.  fl(c - p) is monotone in p, so both shift
// predicates are monotone along a sweep and the points where a shift fires
// are found by bisection instead of visiting every point.
// The points of one sweep where the shifted coordinate changes, with the
// value after each change: a sweep starting from c changes at most a few
// times (a shift down at the first point, a shift up once c - p drops
// below -n/2), so any point's value is a lookup in this short list.
constexpr int MAXEV = 6;
struct SweepEv {
  int nev;
  int ok;
  int j[MAXEV];
  double v[MAXEV];
  double v0;
};
static_assert(7 * sizeof(SweepEv) <= kSweepBytes, "sweep slab too small");
__device__ SweepEv sweep_events(double c, int n, int nh) {
  SweepEv s;
  s.nev = 0;
  s.ok = 1;
  s.v0 = c;
  const double dn = (double)n, dnh = (double)nh;
  int j = 1;
  for (int guard = 0; guard < 16; ++guard) {
    const double p = (double)j - 0.5;
    const double before = c;
    if ((c - p) > dnh) c = c - dn;
    if ((c - p) < -dnh) c = c + dn;
    if (__double_as_longlong(c) != __double_as_longlong(before)) {
      if (s.nev < MAXEV) { s.j[s.nev] = j; s.v[s.nev] = c; ++s.nev; } else s.ok = 0;
    }
    if (j >= n) return s;
    int jn = n + 1;
    const double p1 = (double)(j + 1) - 0.5;
    if ((c - p1) > dnh) {
      jn = j + 1;
    } else if ((c - ((double)n - 0.5)) < -dnh) {
      // the first point m in [j + 1, n] where the shift up fires.  In exact
      // arithmetic that is the first m > c + n/2 + 1/2, and fl(c - p) is
      // within an ulp of c - p, so the FP64 first point lies within two of
      // floor(c + n/2 + 1/2) + 1: scan from two below it with the
      // reference's expression (monotone in m) after checking that the start
      // is not past it; bisect where either check fails (not expected).
      auto up = [&](int m) { return (c - ((double)m - 0.5)) < -dnh; };
      int lo = j + 1, hi = n;
      int m = (int)floor(c + dnh + 0.5) - 1;
      m = m < lo ? lo : (m > hi ? hi : m);
      bool found = false;
      if (m == lo || !up(m - 1)) {
        for (int t = 0; t < 6 && m <= hi; ++t, ++m)
          if (up(m)) { found = true; break; }
        if (!found) lo = m;
      } else {
        hi = m - 1;
      }
      if (!found) {
        while (lo < hi) {
          int mid = (lo + hi) >> 1;
          if (up(mid)) hi = mid; else lo = mid + 1;
        }
        m = lo;
      }
      jn = m;
    }
    if (jn > n) return s;
    j = jn;
  }
  s.ok = 0;
  return s;
}
__device__ __forceinline__ double sweep_value(const SweepEv& s, int jq) {
  double v = s.v0;
  for (int e = 0; e < s.nev; ++e)
    if (s.j[e] <= jq) v = s.v[e];
  return v;
}

// candidate indices (1-based) along one axis: the union, in ascending order,
// of windows of half-width w around c - n, c, c + n, clipped to [1, n].
struct Cands {
  int lo[3], hi[3], cnt;
  __device__ int total() const {
    int t = 0;
    for (int s = 0; s < cnt; ++s) t += hi[s] - lo[s] + 1;
    return t;
  }
  __device__ int at(int t) const {
    for (int s = 0; s < cnt; ++s) {
      int len = hi[s] - lo[s] + 1;
      if (t < len) return lo[s] + t;
      t -= len;
    }
    return -1;
  }
};
__device__ Cands make_cands(double c, int n, double w, bool periodic) {
  Cands cd;
  cd.cnt = 0;
  int L[3], H[3], m = 0;
  for (int s = periodic ? -1 : 0; s <= (periodic ? 1 : 0); ++s) {
    double ctr = c + (double)s * (double)n;
    int lo = (int)floor(ctr - w - 1.0);
    int hi = (int)ceil(ctr + w + 2.0);
    if (lo < 1) lo = 1;
    if (hi > n) hi = n;
    if (lo > hi) continue;
    L[m] = lo; H[m] = hi; ++m;
  }
  // windows are produced in ascending order; merge overlaps
  for (int s = 0; s < m; ++s) {
    if (cd.cnt > 0 && L[s] <= cd.hi[cd.cnt - 1] + 1) {
      if (H[s] > cd.hi[cd.cnt - 1]) cd.hi[cd.cnt - 1] = H[s];
    } else {
      cd.lo[cd.cnt] = L[s]; cd.hi[cd.cnt] = H[s]; ++cd.cnt;
    }
  }
  return cd;
}

constexpr int MAXPLANES = 96;
constexpr int MAXROWS = 640;   // processed rows per particle: (2 (rad + 2) + 1)^2
constexpr int MAXC = 128;  // candidate positions per axis
constexpr int MAXNEAR = 2048;  // fluid nodes within rad + 1.5 of one centre

// Sign decisions of the squared-distance tests of beads_links are taken in
// FP32 when |value| exceeds this margin (the FP32 error is below 1e-4 for
// the offsets involved) and recomputed with the reference's FP64 expression
// otherwise, so the outcome is always the FP64 one.
constexpr float kDecide = 4e-3f;

// beads_links for one particle per block.  Integer outcomes (solid flags,
// link sets) are exactly those of the reference's FP64 loop nest; the link
// fraction alpha is computed in FP64 (alpha_fp32 0: stored FP64; 2: stored
// FP32) or in FP32 (1, the FP32 population path).  The FP32 arithmetic starts
// from offsets node - centre formed in FP64 and rounded once (a difference of
// FP32 coordinates near x = 256 would be off by up to 1.5e-5 lattice units,
// which the bounced populations would inherit), so alpha is good to the FP32
// rounding of the quadratic's terms, about 1e-6.
// The nearest-image history of the in-place sweeps of beads_links
// (partlib.f90:959-985) for every particle: one thread per (particle, axis).
// The y and x sweeps are taken from three start states (the centre, the end
// state of one sweep, the end state of two); the end state is a fixed point
// from the second sweep on unless the centre lies within an ulp of
// n/2 - 1/2, which sweep_ok reports.  FP64 and serial by nature; run for all
// particles at once rather than inside each link block.
__device__ __forceinline__ void k_link_sweeps_body(int bx, int gx, Geometry g, ParticleView pv, LinkSlab ls) {
  const int t = bx * blockDim.x + threadIdx.x;
  if (t >= 3 * pv.npart) return;
  const int p = t / 3, axis = t - 3 * p;
  SweepEv* out = reinterpret_cast<SweepEv*>(static_cast<char*>(ls.sweeps) + (size_t)p * kSweepBytes);
  const double c0 = pv.ypglb[3 * p + (axis == 0 ? 1 : axis == 1 ? 0 : 2)];
  int ok = 1;
  if (!isfinite(c0)) {
    ok = 0;
  } else {
    // The three axes in one instruction stream: y and x take three start
    // states and the fixed-point check (four sweeps), z one sweep; the z
    // lanes run the y and x lanes' four rounds with them and keep only the
    // first, so that a warp pays for four serial sweeps rather than five
    // (FP64 issues at 2 lanes per clock per SM whatever the active lanes).
    const bool xwall = axis == 1 && g.channel;  // no x sweep in the channel
    const int n = axis == 0 ? g.ny : (axis == 1 ? g.nx : g.nz);
    const int nh = axis == 0 ? g.nyh : (axis == 1 ? g.nxh : g.nzh);
    SweepEv* o = out + 3 * axis;
    double c = c0;
    for (int s = 0; s < 4; ++s) {
      const SweepEv e = sweep_events(c, n, nh);
      const double next = sweep_value(e, n);
      if (!xwall) {
        if (axis == 2) {
          if (s == 0) { o[0] = e; ok = e.ok; }
        } else if (s < 3) {
          o[s] = e;
          ok &= e.ok;
        } else if (next != c) {
          ok = 0;
        }
      }
      c = next;
    }
    if (xwall) {
      SweepEv e;
      e.nev = 0; e.ok = 1; e.v0 = c0;
      out[3] = e; out[4] = e; out[5] = e;
    }
  }
  ls.sweep_ok[3 * p + axis] = ok;
}
__global__ void k_link_sweeps(Geometry g, ParticleView pv, LinkSlab ls) {
  k_link_sweeps_body(blockIdx.x, gridDim.x, g, pv, ls);
}

// The reference's FP64 tests of beads_links (partlib.f90:990, 1012), taken
// where the FP32 test is within kDecide of the boundary (rarely).  Out of
// line, so that the compiler keeps them behind their branches: this GPU
// issues FP64 at 2 lanes per clock per SM, and an FP64 instruction costs a
// warp the same whatever its active lanes.  (i, j, k) 1-based, node at
// (i - 1/2, j - 1/2, k - 1/2); the reference's "+ 0.0" offsets are exact
// no-ops here (the point coordinates are positive, and only squares follow).
__device__ __noinline__ bool inside_fp64(int i, int j, int k, double xc, double yc, double zc,
                                         double rad2) {
  const double xx = ((double)i - 0.5) - xc;
  const double yy = ((double)j - 0.5) - yc;
  const double zz = ((double)k - 0.5) - zc;
  const double rr = xx * xx + yy * yy + zz * zz;
  return (rr - rad2) <= 0.0;
}

__device__ __forceinline__ void k_links_body(int bx, int gx, Geometry g, ParticleView pv, int32_t* isnodes,
                                              LinkSlab ls, DevStatus* st, int alpha_fp32) {
  using Scan = cub::BlockScan<int, PB>;
  __shared__ typename Scan::TempStorage scan_tmp;
  __shared__ int plane_k[MAXPLANES];
  __shared__ double plane_z[MAXPLANES];
  __shared__ double plane_zz[MAXPLANES];  // (k - 1/2) - zc of each plane
  __shared__ double yval[3][MAXC];
  __shared__ double yyv[3][MAXC];         // (j - 1/2) - yc per y candidate and start state
  __shared__ float yyvf[3][MAXC];
  __shared__ double xval[3][MAXC];
  __shared__ float xofff[3][MAXC];  // (i - 1/2) - x centre per x candidate, FP64 then rounded
  __shared__ int nplanes;
  __shared__ int row_k[MAXROWS], row_j[MAXROWS];
  __shared__ double row_z[MAXROWS], row_y[MAXROWS];
  __shared__ float row_yy[MAXROWS], row_zz[MAXROWS];
  __shared__ int nrows;
  __shared__ int base;
  __shared__ int fixed_ok;
  __shared__ int near_rc[MAXNEAR];  // fluid nodes within reach: row << 8 | candidate
  __shared__ int nnear;

  const int p = bx;
  if (p >= pv.npart) return;
  const bool channel = g.channel != 0;
  const int tid = threadIdx.x;
  // the block's FP64 constants, formed once (by thread 0) rather than by
  // every warp: FP64 instructions are the scarce issue slots of this GPU
  __shared__ double s_par[5];  // radp2, rad2, x0, y0, z0
  __shared__ float s_parf[2];  // rad2 and the squared reach in FP32
  __shared__ int s_finite;
  if (tid == 0) {
    nplanes = 0; nrows = 0; base = 0; fixed_ok = 1; nnear = 0;
    const double rad = pv.rad;
    s_par[0] = rad * 1.0 + 2.0;
    s_par[1] = (rad * 1.0) * (rad * 1.0);
    s_parf[0] = (float)s_par[1];
    // only nodes within rad + sqrt(2) of the centre can be solid or own a link
    s_parf[1] = (float)((rad + 1.5) * (rad + 1.5)) + 0.05f;
    for (int a = 0; a < 3; ++a) s_par[2 + a] = pv.ypglb[3 * p + a] * 1.0;
    s_finite = isfinite(s_par[2]) && isfinite(s_par[3]) && isfinite(s_par[4]);
  }
  __syncthreads();
  const double radp2 = s_par[0], rad2 = s_par[1];
  const float rad2f = s_parf[0], reachf = s_parf[1];
  const double x0 = s_par[2], y0 = s_par[3], z0 = s_par[4];
  if (!s_finite) {
    if (tid == 0) {
      ls.count[p] = 0;
      raise_error(st, LBM_ERR_NONFINITE, p);
    }
    return;
  }
  // Sweep event lists (k_link_sweeps) for the start states of the y sweep
  // (plane 0 starts at y0, plane 1 at Y1 = end of plane 0's sweep, later
  // planes at Y2) and of the x sweep (rows likewise: x0, X1, X2), and for the
  // single z sweep.
  __shared__ SweepEv sev[7];  // 0..2: y states, 3..5: x states, 6: z
  if (tid < 7) sev[tid] = reinterpret_cast<const SweepEv*>(
      static_cast<const char*>(ls.sweeps) + (size_t)p * kSweepBytes)[tid];
  if (tid == 0) {
    const int32_t* ok = ls.sweep_ok + 3 * p;
    if (!(ok[0] && ok[1] && ok[2])) fixed_ok = 0;
  }
  // candidate windows of the three axes, computed once for the block
  __shared__ Cands cands[3];
  if (tid == 0) cands[0] = make_cands(y0, g.ny, radp2, true);
  else if (tid == 32) cands[1] = make_cands(x0, g.nx, radp2, !channel);
  else if (tid == 64) cands[2] = make_cands(z0, g.nz, radp2, true);
  __syncthreads();
  const Cands& cy = cands[0];
  const Cands& cx = cands[1];
  const int ty = min(cy.total(), MAXC);
  const int tx = min(cx.total(), MAXC);
  for (int t = tid; t < 3 * MAXC; t += PB) {
    int s = t / MAXC, c = t % MAXC;
    if (c < ty) {
      const double yc = sweep_value(sev[s], cy.at(c));
      yval[s][c] = yc;
      const double yy0 = ((double)cy.at(c) - 0.5) - yc;
      yyv[s][c] = yy0;
      yyvf[s][c] = (float)yy0;
    }
    if (c < tx) {
      double v = channel ? x0 : sweep_value(sev[3 + s], cx.at(c));
      xval[s][c] = v;
      xofff[s][c] = (float)(((double)cx.at(c) - 0.5) - v);
    }
  }
  if (tid == 0 && (cy.total() > MAXC || cx.total() > MAXC)) fixed_ok = 0;
  __syncthreads();

  // ---- planes: k with |zz0| <= radp2, zc from the k-sweep starting at z0
  const Cands& cz = cands[2];
  int tz = cz.total();
  for (int c0 = 0; c0 < tz; c0 += PB) {
    int t = c0 + tid;
    int k = -1;
    double zc = 0.0, zz0 = 0.0;
    bool take = false;
    if (t < tz) {
      k = cz.at(t);
      zc = sweep_value(sev[6], k);
      double zpnt = (double)k - 0.5;
      zz0 = zpnt - zc;
      take = fabs(zz0) <= radp2;
    }
    int pos, tot;
    Scan(scan_tmp).ExclusiveSum(take ? 1 : 0, pos, tot);
    __syncthreads();
    if (take && nplanes + pos < MAXPLANES) {
      plane_k[nplanes + pos] = k;
      plane_z[nplanes + pos] = zc;
      plane_zz[nplanes + pos] = zz0;
    }
    __syncthreads();
    if (tid == 0) nplanes = min(nplanes + tot, MAXPLANES);
    __syncthreads();
  }

  // ---- rows: per plane (in k order), j with the exact y condition
  int tpairs = nplanes * ty;
  for (int c0 = 0; c0 < tpairs; c0 += PB) {
    int t = c0 + tid;
    bool take = false;
    int k = 0, j = 0, pi = 0, c = 0;
    if (t < tpairs) {
      // the offsets of the row's plane and y candidate come from the tables
      // above (the same values; the FP64 work done once per plane and
      // candidate rather than per pair)
      pi = t / ty;
      c = t - pi * ty;
      j = cy.at(c);
      k = plane_k[pi];
      const double zz0 = plane_zz[pi], yy0 = yyv[min(pi, 2)][c];
      take = channel ? (sqrt(yy0 * yy0 + zz0 * zz0) <= radp2) : (fabs(yy0) <= radp2);
    }
    int pos, tot;
    Scan(scan_tmp).ExclusiveSum(take ? 1 : 0, pos, tot);
    __syncthreads();
    if (take && nrows + pos < MAXROWS) {
      int w = nrows + pos;
      row_k[w] = k; row_j[w] = j; row_z[w] = plane_z[pi]; row_y[w] = yval[min(pi, 2)][c];
      row_yy[w] = yyvf[min(pi, 2)][c]; row_zz[w] = (float)plane_zz[pi];
    }
    __syncthreads();
    if (tid == 0) nrows = min(nrows + tot, MAXROWS);
    __syncthreads();
  }

  // ---- phase 1: nodes of every processed row within reach of the sphere;
  // solid nodes are flagged, fluid ones kept (in row, then x order) for
  // phase 2.  One thread per row; a block scan of the per-row counts places
  // each row's nodes.
  // class of node (row r, x candidate ci): 0 out of reach, 1 solid, 2 fluid
  auto node_class = [&](int r, int ci) -> int {
    const int i = cx.at(ci);
    const float xxf = xofff[min(r, 2)][ci];
    const float yyf = row_yy[r], zzf = row_zz[r];
    const float rr0f = xxf * xxf + yyf * yyf + zzf * zzf;
    if (!(rr0f <= reachf)) return 0;
    const float d0 = rr0f - rad2f;
    if (d0 < -kDecide) return 1;
    if (d0 > kDecide) return 2;
    return inside_fp64(i, row_j[r], row_k[r], xval[min(r, 2)][ci], row_y[r], row_z[r], rad2) ? 1
                                                                                             : 2;
  };
  for (int r0 = 0; r0 < nrows; r0 += PB) {
    const int r = r0 + tid;
    int cnt = 0;
    if (r < nrows) {
      const int j = row_j[r], k = row_k[r];
      for (int ci = 0; ci < tx; ++ci) {
        const int cl = node_class(r, ci);
        if (cl == 1) {
          const int i = cx.at(ci);
          long long node = (long long)(i - 1) + (long long)g.nx * ((j - 1) + (long long)g.ny * (k - 1));
          atomicMax(&isnodes[node], p);
          uint32_t* mask = const_cast<uint32_t*>(solid_mask(isnodes, g));
          atomicOr(&mask[((size_t)(k - 1) * g.ny + (j - 1)) * g.sw + ((i - 1) >> 5)],
                   1u << ((i - 1) & 31));
        } else if (cl == 2) {
          ++cnt;
        }
      }
    }
    int pos, tot;
    Scan(scan_tmp).ExclusiveSum(cnt, pos, tot);
    if (cnt) {
      int w = nnear + pos;
      for (int ci = 0; ci < tx; ++ci)
        if (node_class(r, ci) == 2) {
          if (w < MAXNEAR) near_rc[w] = (r << 8) | ci;
          ++w;
        }
    }
    __syncthreads();
    if (tid == 0) {
      if (nnear + tot > MAXNEAR) fixed_ok = 0;
      nnear = min(nnear + tot, MAXNEAR);
    }
    __syncthreads();
  }

  // ---- phase 2: one thread per fluid near node tests its 18 directions.
  // Within each chunk of PB near nodes the links are written direction by
  // direction (ipop, then node order), so that the bounce-back kernels that
  // walk the list read and write neighbouring x nodes of one population
  // array together.  Offsets come from warp ballots per direction and one
  // warp-wide scan of the (direction, warp) counts.
  constexpr int NW = PB / 32;
  constexpr int NCNT = 18 * NW;
  constexpr int PER_LANE = (NCNT + 31) / 32;
  __shared__ int woff[NCNT];
  __shared__ int chunk_links;
  __shared__ int16_t link_src[PB * 18];  // per link of the chunk: near node (local) << 5 | ipop
  const int warp = tid >> 5, lane = tid & 31;
  const unsigned lane_lt = (1u << lane) - 1u;
  int32_t* code = ls.code + (long long)p * ls.cap;
  double* alph = ls.alpha + (long long)p * ls.cap;
  float* alph32 = reinterpret_cast<float*>(alph);
  for (int n0 = 0; n0 < nnear; n0 += PB) {
    const int idx = n0 + tid;
    unsigned mask = 0;
    int r = 0, ci = 0, i = 0;
    float xxf = 0.f, yyf = 0.f, zzf = 0.f;
    if (idx < nnear) {
      const int rc = near_rc[idx];
      r = rc >> 8;
      ci = rc & 255;
      i = cx.at(ci);
      xxf = xofff[min(r, 2)][ci];
      yyf = row_yy[r];
      zzf = row_zz[r];
#pragma unroll
      for (int ipop = 1; ipop < NPOP; ++ipop) {
        const float ax = xxf + (float)cix(ipop), ay = yyf + (float)ciy(ipop), az = zzf + (float)ciz(ipop);
        const float d1 = ax * ax + ay * ay + az * az - rad2f;
        bool link;
        if (d1 < -kDecide) link = true;
        else if (d1 > kDecide) link = false;
        else
          link = inside_fp64(i + cix(ipop), row_j[r] + ciy(ipop), row_k[r] + ciz(ipop),
                             xval[min(r, 2)][ci], row_y[r], row_z[r], rad2);
        if (link) mask |= 1u << ipop;
      }
    }
#pragma unroll
    for (int q = 0; q < 18; ++q) {
      const unsigned bal = __ballot_sync(0xffffffffu, (mask >> (q + 1)) & 1u);
      if (lane == 0) woff[q * NW + warp] = __popc(bal);
    }
    __syncthreads();
    if (warp == 0) {
      // exclusive scan of the NCNT counts, PER_LANE consecutive entries a lane
      int v[PER_LANE], sum = 0;
#pragma unroll
      for (int e = 0; e < PER_LANE; ++e) {
        const int t = lane * PER_LANE + e;
        v[e] = t < NCNT ? woff[t] : 0;
        sum += v[e];
      }
      int incl = sum;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += o;
      }
      int run = incl - sum;
#pragma unroll
      for (int e = 0; e < PER_LANE; ++e) {
        const int t = lane * PER_LANE + e;
        if (t < NCNT) woff[t] = run;
        run += v[e];
      }
      if (lane == 31) chunk_links = incl;
    }
    __syncthreads();
    {
      const int j = row_j[r], k = row_k[r];
      const long long node =
          (long long)(i - 1) + (long long)g.nx * ((j - 1) + (long long)g.ny * (k - 1));
#pragma unroll 1
      for (int q = 0; q < 18; ++q) {
        const int ipop = q + 1;
        const bool has = (mask >> ipop) & 1u;
        const unsigned bal = __ballot_sync(0xffffffffu, has);
        if (!has) continue;
        const int l = woff[q * NW + warp] + __popc(bal & lane_lt);
        link_src[l] = (int16_t)((tid << 5) | ipop);
        if (base + l < ls.cap) code[base + l] = (int32_t)(node * 32 + ipop);
      }
    }
    __syncthreads();
    // link fractions, one thread per link of the chunk (all lanes busy)
    for (int l = tid; l < chunk_links; l += PB) {
      const int w = base + l;
      if (w >= ls.cap) break;
      const int src = link_src[l];
      const int ipop = src & 31;
      const int rc = near_rc[n0 + (src >> 5)];
      const int lr = rc >> 8, lci = rc & 255;
      const int li = cx.at(lci);
      const int ix = cix(ipop), iy = ciy(ipop), iz = ciz(ipop);
      const bool diag = (ix * ix + iy * iy + iz * iz) == 2;
      // partlib.f90:1016-1023 with aa = |x0 - x1|^2 = |c|^2 (1 or 2) and
      // bb = x1.(x0 - x1) = -x1.c taken exactly: the same root without the
      // cancellation in the reference's aa and without divisions
      if (alpha_fp32 == 1) {
        const float xf = xofff[min(lr, 2)][lci] + (float)ix;
        const float yf = row_yy[lr] + (float)iy, zf = row_zz[lr] + (float)iz;
        const float cc = xf * xf + yf * yf + zf * zf - rad2f;
        const float bb = -(xf * (float)ix + yf * (float)iy + zf * (float)iz);
        const float a0 = diag ? 0.5f * bb : bb;
        const float ca = diag ? 0.5f * cc : cc;
        const float a1 = sqrtf(fmaxf(a0 * a0 - ca, 0.0f));
        alph32[w] = 1.0f - (-a0 + a1);
      } else {
        // the components of c are +-1 or 0: c . x1 is selects and one add
        auto pick = [](int c, double v) { return flip_if(c < 0, v); };
        const int lj = row_j[lr], lk = row_k[lr];
        const double xx1 = (double)(li + ix) - 0.5 - xval[min(lr, 2)][lci];
        const double yy1 = (double)(lj + iy) - 0.5 - row_y[lr];
        const double zz1 = (double)(lk + iz) - 0.5 - row_z[lr];
        double bb;
        if (ix == 0) bb = iy == 0 ? pick(iz, zz1) : (iz == 0 ? pick(iy, yy1) : pick(iy, yy1) + pick(iz, zz1));
        else bb = iy != 0 ? pick(ix, xx1) + pick(iy, yy1)
                          : (iz != 0 ? pick(ix, xx1) + pick(iz, zz1) : pick(ix, xx1));
        // the reference's bb is -(c . x1); its negation folded into a0
        const double cc = fma(xx1, xx1, fma(yy1, yy1, fma(zz1, zz1, -rad2)));
        const double a0 = diag ? -0.5 * bb : flip_if(true, bb);
        const double ca = diag ? 0.5 * cc : cc;
        // max(disc, 0) by the sign bit (an integer select)
        const double disc = fma(a0, a0, -ca);
        const double a1 = sqrt(__double_as_longlong(disc) < 0 ? 0.0 : disc);
        const double a = 1.0 - (-a0 + a1);
        if (alpha_fp32 == 2) alph32[w] = (float)a;  // FP32 slab, FP64 arithmetic
        else alph[w] = a;
      }
    }
    __syncthreads();
    if (tid == 0) base += chunk_links;
    __syncthreads();
  }
  if (tid == 0) {
    ls.count[p] = min(base, ls.cap);
    if (base > ls.cap) raise_error(st, LBM_ERR_CAPACITY, p);
    if (nplanes >= MAXPLANES || nrows >= MAXROWS) raise_error(st, LBM_ERR_CAPACITY, p);
    if (!fixed_ok) raise_error(st, LBM_ERR_STATE, p);
  }
}
__global__ void __launch_bounds__(PB) k_links(Geometry g, ParticleView pv, int32_t* isnodes,
                                              LinkSlab ls, DevStatus* st, int alpha_fp32) {
  k_links_body(blockIdx.x, gridDim.x, g, pv, isnodes, ls, st, alpha_fp32);
}

// running sum: plain FP64, or FP32 with Kahan compensation (FP32 path)
template <typename T>
struct Acc {
  double s = 0.0;
  __device__ void add(double x) { s += x; }
  __device__ void add_prod(double a, double b) { s = fma(a, b, s); }
  __device__ double value() const { return s; }
};
template <>
struct Acc<float> {
  float s = 0.f, c = 0.f;
  __device__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ void add_prod(float a, float b) { add(a * b); }
  __device__ double value() const { return (double)s - (double)c; }
};

// 1 / x for x in [1/2, 3] (the link-fraction denominators of the bounce-back).
// FP64: Newton-Raphson reciprocal iteration r <- r + r (1 - x r) from a
// single-precision seed; each step squares the relative error, so two steps
// take the seed's 2^-22 below the FP64 rounding.  On this GPU FP64 issues at
// a small fraction of the FP32 rate, and the iteration is 4 FMAs.
__device__ __forceinline__ double recip_link(double x) {
  const float xf = __double2float_rn(x);
  float r0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(xf));
  double r = (double)r0;
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}
__device__ __forceinline__ float recip_link(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double fma_r(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_r(float a, float b, float c) { return fmaf(a, b, c); }

// a stored population: FP64 populations are 64-bit fixed point while
// g.pop_fixed is set (between fused steps of the FP64 plain path)
template <typename T>
__device__ __forceinline__ T ld_pop(const Geometry& g, const T* f, long long idx) {
  if constexpr (sizeof(T) == 8) {
    if (g.pop_fixed) return pop_from_fixed(reinterpret_cast<const long long*>(f)[idx]);
  }
  return f[idx];
}
template <typename T>
__device__ __forceinline__ void st_pop(const Geometry& g, T* f, long long idx, T v, DevStatus* st,
                                       int where) {
  if constexpr (sizeof(T) == 8) {
    if (g.pop_fixed) {
      long long w;
      if (!pop_to_fixed(v, w)) raise_error(st, LBM_ERR_NONFINITE, where);
      reinterpret_cast<long long*>(f)[idx] = w;
      return;
    }
  }
  f[idx] = v;
}

// post-collision population q at node (i, j, k) (0-based) in either layout.
// pushed: the fused kernel has already moved it to its streaming target
// (or bounced it back in place at a channel wall).
template <typename T>
__device__ __forceinline__ T read_post(const Geometry& g, const T* f, int pushed, int q, int i,
                                       int j, int k) {
  // 32-bit element indices: 19 N < 2^31 (N < 2^26 is enforced)
  const int N = (int)g.N;
  const int n = i + g.nx * (j + g.ny * k);
  if (!pushed) return ld_pop(g, f, q * N + n);
  int it = i + cix(q);
  if (g.channel && (it < 0 || it >= g.nx)) return ld_pop(g, f, ipopp(q) * N + n);
  it = wrapi(it, g.nx);
  const int jt = wrapi(j + ciy(q), g.ny), kt = wrapi(k + ciz(q), g.nz);
  return ld_pop(g, f, q * N + it + g.nx * (jt + g.ny * kt));
}

// threads per particle block of the bounce-back: 128 threads leave fewer
// idle lanes in the last pass over a particle's ~1000 links than 256, and
// eight such blocks fit an SM (the batched kernel uses the same count, so a
// box's force sums run in the same order alone and in a batch)
template <typename T>
constexpr int bounce_threads() { return 128; }

// beads_collision for one particle per block of NT threads: every link
// computes the bounced population f9 (stored per link) and its momentum
// exchange.
template <typename T, int NT>
__device__ __forceinline__ void k_bounce_body(int bx, int gx, Geometry g, ParticleView pv, const T* f, int pushed,
                                               const int32_t* __restrict__ isnodes, LinkSlab ls,
                                               double* fHIp, double* torqp) {
  const int p = bx;
  if (p >= pv.npart) return;
  const int cnt = ls.count[p];
  const int32_t* code = ls.code + (long long)p * ls.cap;
  // link fractions and bounced populations are stored in the population
  // precision (FP32 slabs reuse the first half of the FP64 arrays)
  const T* alph = reinterpret_cast<const T*>(ls.alpha + (long long)p * ls.cap);
  T* f9s = reinterpret_cast<T*>(ls.f9 + (long long)p * ls.cap);
  // per-link arithmetic in the population precision R (FP64 plain path,
  // FP32 shifted path); each thread's partial force/torque sums are
  // compensated (FP32) or plain FP64, the block sums are FP64
  using R = T;
  Acc<T> acc6[6];
  // the particle's velocities in the arithmetic precision and the first
  // tabulated coordinate per axis, formed once by thread 0 (conversions and
  // roundings of FP64 values issue on the FP64 pipe, and cost a warp the same
  // whatever its active lanes)
  __shared__ R s_wo[6];
  __shared__ int s_lo[4];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      s_wo[a] = R(pv.wp[3 * p + a]);
      s_wo[3 + a] = R(pv.omgp[3 * p + a]);
      s_lo[a] = (int)floor((double)pv.ypglb[3 * p + a]) - (kBounceSpan / 2);
    }
    // the link nodes lie within rad + sqrt(2) of the centre: the entries
    // kBounceSpan / 2 +- (ceil(rad) + 3) of the table cover them
    s_lo[3] = min((int)ceil(pv.rad) + 3, kBounceSpan / 2 - 1);
  }
  __syncthreads();
  const R w1 = s_wo[0], w2 = s_wo[1], w3 = s_wo[2];
  const R omg1 = s_wo[3], omg2 = s_wo[4], omg3 = s_wo[5];
  const R xc0 = R(0), yc0 = R(0), zc0 = R(0);  // (unused by delta)
  const bool channel = g.channel != 0;
  const uint32_t* mask = solid_mask(isnodes, g);
  // Per axis, the offset d = pnt - c of the link point pnt = i + 1/2 from the
  // image c of the centre nearest to it depends on the node's coordinate i
  // alone: tabulate it once per particle for the coordinates around the
  // centre that links reach (same operations as per link, so the same
  // values); links outside the table compute it directly.  Per direction,
  // c_q . w.
  __shared__ R tdel[3][kBounceSpan];
  __shared__ R tcw[NPOP];
  // c_a v with c_a in {-1, 0, 1}: exact, so selected rather than multiplied
  auto sel = [](int c, R v) { return c == 0 ? R(0) : flip_if(c < 0, v); };
  const int lo[3] = {s_lo[0], s_lo[1], s_lo[2]};
  const int dlo = kBounceSpan / 2 - s_lo[3], dhi = kBounceSpan / 2 + s_lo[3];
  {
    // selects rather than arrays indexed by a, which would live in local memory
    const int span = dhi - dlo + 1;
    for (int t = threadIdx.x; t < 3 * span; t += NT) {
      const int a = t / span, d = dlo + (t - a * span);
      const bool periodic = !(channel && a == 0);
      // in FP64 whatever R: an FP32 centre near x = 256 is off by 1.5e-5
      const double cen = pv.ypglb[3 * p + a];
      const int n = a == 0 ? g.nx : (a == 1 ? g.ny : g.nz);
      const int nh = a == 0 ? g.nxh : (a == 1 ? g.nyh : g.nzh);
      int i = (a == 0 ? lo[0] : (a == 1 ? lo[1] : lo[2])) + d;
      if (periodic) i = ((i % n) + n) % n;
      const double pnt = (double)(i + 1) - 0.5;
      tdel[a][d] = R(pnt - (periodic ? near_img_t<double>(cen, pnt, n, nh) : cen));
    }
    if (threadIdx.x < NPOP) {
      const int q = threadIdx.x;
      tcw[q] = sel(cix(q), w1) + sel(ciy(q), w2) + sel(ciz(q), w3);
    }
    __syncthreads();
  }
  auto delta = [&](int a, int i, R, int n, int nhalf, bool periodic) -> R {
    int d = i - lo[a];
    if (periodic) d = d < 0 ? d + n : (d >= n ? d - n : d);
    if (d >= dlo && d <= dhi) return tdel[a][d];
    const double cen = pv.ypglb[3 * p + a];
    const double pnt = (double)(i + 1) - 0.5;
    return R(pnt - (periodic ? near_img_t<double>(cen, pnt, n, nhalf) : cen));
  };
  // cb db - cc dc for cb, cc in {-1, 0, 1}: one add at most
  auto cross = [](int cb, R db, int cc, R dc) -> R {
    const R u = cb == 0 ? R(0) : flip_if(cb < 0, db);
    if (cc == 0) return u;
    const R v = flip_if(cc < 0, dc);
    return cb == 0 ? flip_if(true, v) : u - v;
  };
  for (int l = threadIdx.x; l < cnt; l += NT) {
    // 32-bit decode: node < 2^26
    const int cd = code[l];
    const int ipop = cd & 31;
    const int node = cd >> 5;
    const int r = node / g.nx;
    const int i = node - r * g.nx;
    const int k = r / g.ny, j = r - k * g.ny;
    const R alpha = alph[l];
    const int ipp = ipopp(ipop);
    const int ix = cix(ipop), iy = ciy(ipop), iz = ciz(ipop);
    int im1 = i - ix, im2 = i - 2 * ix;
    const int jm1 = wrapi(j - iy, g.ny), km1 = wrapi(k - iz, g.nz);
    const int jm2 = wrapi(j - 2 * iy, g.ny), km2 = wrapi(k - 2 * iz, g.nz);
    bool out1 = false, out2 = false;
    if (channel) {
      out1 = im1 < 0 || im1 >= g.nx;
      out2 = im2 < 0 || im2 >= g.nx;
    } else {
      im1 = wrapi(im1, g.nx);
      im2 = wrapi(im2, g.nx);
    }
    // The reference's lever arm is r = d + alpha c (the boundary point);
    // every quantity it enters is a product with c: the wall velocity
    // c . (w + omega x r) = c . w + omega . (r x c) and the torque
    // dff (r x c), and r x c = d x c.  So the per-link arithmetic needs only
    // e = d x c, which for c in {-1, 0, 1}^3 is selects and one add.
    const R dx = delta(0, i, xc0, g.nx, g.nxh, !channel);
    const R dy = delta(1, j, yc0, g.ny, g.nyh, true);
    const R dz = delta(2, k, zc0, g.nz, g.nzh, true);
    const R ex = cross(iz, dy, iy, dz);
    const R ey = cross(ix, dz, iz, dx);
    const R ez = cross(iy, dx, ix, dy);
    const R uwpro = fma_r(omg1, ex, fma_r(omg2, ey, fma_r(omg3, ez, tcw[ipop])));
    const R ff1 = R(read_post(g, f, pushed, ipop, i, j, k));
    // The five interpolation cases of beads_collision (B/partlib.f90:1439-1536)
    // as f9 = c1 ff1 + c2 ff2 + c3 ff3 - 6 w c4 (c . u_w), with the same
    // populations read and one division (for alpha > 1/2) shared by its two
    // cases, so that a warp with mixed cases evaluates one formula:
    //   alpha <= 1/2: ff2, ff3 = f(q) at x - c, x - 2c
    //     x - c solid:  c1 = 1
    //     x - 2c solid: c1 = 2 alpha, c2 = 1 - 2 alpha
    //     else:         c1 = alpha (1 + 2 alpha), c2 = 1 - 4 alpha^2,
    //                   c3 = -alpha (1 - 2 alpha)
    //   alpha > 1/2: ff2, ff3 = f(qbar) at x, x - c;  c4 = c1
    //     x - c solid:  c1 = 1 / (2 alpha), c2 = 1 - c1
    //     else:         c1 = 1 / (alpha (2 alpha + 1)),
    //                   c2 = (2 alpha - 1)(2 alpha + 1) c1, c3 = 1 - c1 - c2
    // alpha <= 1/2 on the bit patterns (an integer compare; the same outcome
    // for every alpha but a NaN with the sign bit set)
    bool low;
    if constexpr (sizeof(R) == 8) low = __double_as_longlong(alpha) <= __double_as_longlong(0.5);
    else low = __float_as_int(alpha) <= __float_as_int(0.5f);
    int ibm1 = 2, ibm2 = 2;
    if (!out1) ibm1 = is_solid(mask, g, km1 * g.ny + jm1, im1) ? 1 : -1;
    if (low && !out2) ibm2 = is_solid(mask, g, km2 * g.ny + jm2, im2) ? 1 : -1;
    const bool s1 = ibm1 > 0;
    const bool s2 = low && !s1 && ibm2 > 0;
    R ff2 = R(0), ff3 = R(0);
    if (low) {
      if (!s1) ff2 = R(read_post(g, f, pushed, ipop, im1, jm1, km1));
      if (!s1 && !s2) ff3 = R(read_post(g, f, pushed, ipop, im2, jm2, km2));
    } else {
      ff2 = R(read_post(g, f, pushed, ipp, i, j, k));
      if (!s1) ff3 = R(read_post(g, f, pushed, ipp, im1, jm1, km1));
    }
    const R t2 = alpha + alpha;
    const R opt = R(1.0) + t2;             // 1 + 2 alpha
    const R omt = R(1.0) - t2;             // 1 - 2 alpha
    const R xa = alpha * opt;              // alpha (1 + 2 alpha)
    const R y4 = omt * opt;                // 1 - 4 alpha^2
    const R rc = recip_link(low ? R(1.0) : (s1 ? alpha : xa));
    R c1, c2, c3, c4;
    if (low) {
      c1 = s1 ? R(1.0) : (s2 ? t2 : xa);
      c2 = s1 ? R(0.0) : (s2 ? omt : y4);
      c3 = (s1 || s2) ? R(0.0) : -alpha * omt;
      c4 = R(1.0);
    } else {
      c1 = s1 ? R(0.5) * rc : rc;
      c2 = s1 ? R(1.0) - c1 : -y4 * rc;
      c3 = s1 ? R(0.0) : R(1.0) - c1 - c2;
      c4 = c1;
    }
    const R k6 = ipop <= 6 ? R(6.0 / 18.0) : R(6.0 / 36.0);
    const R f9 = fma_r(c1, ff1, fma_r(c2, ff2, fma_r(c3, ff3, -(k6 * c4) * uwpro)));
    f9s[l] = f9;
    const R dff = ff1 + f9;
    if (ix) acc6[0].add(flip_if(ix < 0, dff));
    if (iy) acc6[1].add(flip_if(iy < 0, dff));
    if (iz) acc6[2].add(flip_if(iz < 0, dff));
    acc6[3].add_prod(dff, ex);
    acc6[4].add_prod(dff, ey);
    acc6[5].add_prod(dff, ez);
  }
  if constexpr (sizeof(T) == 4) {
    // per warp: exact two-sum tree of the compensated FP32 partial sums;
    // across warps: FP64 in a fixed order (deterministic)
    __shared__ double wsum[6][NT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      float hi = acc6[c].s, lo = -acc6[c].c;
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) {
        const float oh = __shfl_down_sync(0xffffffffu, hi, d);
        const float ol = __shfl_down_sync(0xffffffffu, lo, d);
        const float sh = hi + oh;            // two-sum of the high parts
        const float bp = sh - hi;
        const float err = (hi - (sh - bp)) + (oh - bp);
        hi = sh;
        lo = lo + ol + err;
      }
      if (lane == 0) wsum[c][warp] = (double)hi + (double)lo;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
      const int c = threadIdx.x;
      double s = 0.0;
      for (int w = 0; w < NT / 32; ++w) s += wsum[c][w];
      if (c < 3) fHIp[3 * p + c] = s; else torqp[3 * p + c - 3] = s;
    }
  } else {
    // the threads' six partial sums through shared memory; one warp per
    // component adds NT / 32 of them a lane, then the lanes by an xor
    // butterfly (a fixed order: deterministic)
    __shared__ double part[6][NT];
#pragma unroll
    for (int c = 0; c < 6; ++c) part[c][threadIdx.x] = acc6[c].value();
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = warp; c < 6; c += NT / 32) {
      double s = part[c][lane];
#pragma unroll
      for (int w = 1; w < NT / 32; ++w) s += part[c][lane + 32 * w];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) {
        if (c < 3) fHIp[3 * p + c] = s; else torqp[3 * p + c - 3] = s;
      }
    }
  }
}
template <typename T>
// (64 registers: eight 128-thread blocks per SM, so that the 1000 particle
// blocks of the workload take one wave)
__global__ void __launch_bounds__(bounce_threads<T>(), 8) k_bounce(Geometry g, ParticleView pv, const T* f, int pushed,
                                               const int32_t* __restrict__ isnodes, LinkSlab ls,
                                               double* fHIp, double* torqp) {
  k_bounce_body<T, bounce_threads<T>()>(blockIdx.x, gridDim.x, g, pv, f, pushed, isnodes, ls, fHIp, torqp);
}

// the bounce-back stores of beads_collision: f(ipp, x + c) = f9
// (B/partlib.f90:1605-1621).  In the pushed layout that pre-streaming slot
// already sits at its streaming target, the fluid node x itself.
template <typename T>
__device__ __forceinline__ void k_bounce_store_body(int bx, int gx, Geometry g, ParticleView pv, T* f, int pushed,
                                                     LinkSlab ls, DevStatus* st = nullptr) {
  // particles bx, bx + gx, ...
  for (int p = bx; p < pv.npart; p += gx) {
  const int cnt = ls.count[p];
  const int32_t* code = ls.code + (long long)p * ls.cap;
  const T* f9s = reinterpret_cast<const T*>(ls.f9 + (long long)p * ls.cap);
  for (int l = threadIdx.x; l < cnt; l += PB) {
    const int cd = code[l];
    const int ipop = cd & 31;
    const int node = cd >> 5;
    const int ipp = ipopp(ipop);
    const int r = node / g.nx;
    const int i = node - r * g.nx;
    if (pushed) {
      int it = i + cix(ipop);
      if (g.channel && (it < 0 || it >= g.nx)) continue;
      st_pop(g, f, ipp * g.N + node, f9s[l], st, p);
    } else {
      const int k = r / g.ny, j = r - k * g.ny;
      int it = i + cix(ipop);
      if (g.channel && (it < 0 || it >= g.nx)) continue;
      it = wrapi(it, g.nx);
      int jt = wrapi(j + ciy(ipop), g.ny), kt = wrapi(k + ciz(ipop), g.nz);
      st_pop(g, f, ipp * g.N + (long long)it + (long long)g.nx * (jt + (long long)g.ny * kt), f9s[l], st, p);
    }
  }
  }
}
template <typename T>
__global__ void __launch_bounds__(PB) k_bounce_store(Geometry g, ParticleView pv, T* f, int pushed,
                                                     LinkSlab ls, DevStatus* st) {
  k_bounce_store_body<T>(blockIdx.x, gridDim.x, g, pv, f, pushed, ls, st);
}

// beads_lubforce, one warp per particle.  Contributions to particle p are
// accumulated in ascending partner id, the order in which the reference's
// pair loop (id ascending, jj > id) reaches them.  Pairs farther apart than
// the lubrication range contribute exact zeros in the reference; the warp
// finds the near partners with a single-precision range test (wide margin)
// and lane 0 adds their FP64 contributions in id order.
// An FP64 value as FP32, truncated (relative error below 2^-23), by integer
// operations on its bits: a double-to-float conversion issues on the FP64
// pipe, which this GPU runs at 2 lanes per clock per SM, and the pair
// prefilters below convert every pair's coordinates.  Magnitudes below
// 2^-126 give 0, magnitudes beyond the FP32 range the largest float (only
// coordinates within a box are converted, |v| < 2^30).
__device__ __forceinline__ float f32_trunc(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
  if (e <= 0) return 0.0f;
  if (e >= 255) return __uint_as_float((hi & 0x80000000u) | 0x7f7fffffu);  // (not a box coordinate)
  return __uint_as_float((hi & 0x80000000u) | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) |
                         (lo >> 29));
}

// FP32 prefilter of a particle pair: the centres within lim per axis and in
// distance, nearest image (a margin of a lattice unit over the exact FP64
// test that follows, far above the FP32 error of the coordinates)
__device__ __forceinline__ bool near_pair(const Geometry& g, const double* y, int p, int q,
                                          float lim) {
  float dx = fabsf(f32_trunc(y[3 * q]) - f32_trunc(y[3 * p]));
  float dy = fabsf(f32_trunc(y[3 * q + 1]) - f32_trunc(y[3 * p + 1]));
  float dz = fabsf(f32_trunc(y[3 * q + 2]) - f32_trunc(y[3 * p + 2]));
  if (!g.channel) dx = fminf(dx, (float)g.nx - dx);
  dy = fminf(dy, (float)g.ny - dy);
  dz = fminf(dz, (float)g.nz - dz);
  return dx <= lim && dy <= lim && dz <= lim && dx * dx + dy * dy + dz * dz <= lim * lim;
}

__device__ __forceinline__ void k_lubforce_body(int bx, int gx, Geometry g, int npart, PartParams pp, MoveState ms) {
  const int p = (bx * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (p >= npart) return;
  const bool channel = g.channel != 0;
  const double rad = pp.rad, mingap = pp.mingap;
  const double dist0 = 2.0 * rad + mingap;
  const float lim = (float)(dist0 + 1.0);
  const double* y = ms.ypglb;
  double acc[3] = {0.0, 0.0, 0.0};
  for (int q0 = 0; q0 < npart; q0 += 32) {
    const int qq = q0 + lane;
    const bool cand = qq < npart && qq != p && near_pair(g, y, p, qq, lim);
    unsigned m = __ballot_sync(0xffffffffu, cand);
    if (lane != 0) continue;
    while (m) {
      const int q = q0 + __ffs(m) - 1;
      m &= m - 1;
      // the pair as the reference evaluates it: centre "c" is the lower id
      const int id = min(p, q), jj = max(p, q);
      double xc = y[3 * id], yc = y[3 * id + 1], zc = y[3 * id + 2];
      double xb = y[3 * jj], yb = y[3 * jj + 1], zb = y[3 * jj + 2];
      if (!channel) xb = near_img(xb, xc, g.nx, g.nxh);
      yb = near_img(yb, yc, g.ny, g.nyh);
      zb = near_img(zb, zc, g.nz, g.nzh);
      double dxij = xc - xb, dyij = yc - yb, dzij = zc - zb;
      double dist = sqrt(dxij * dxij + dyij * dyij + dzij * dzij);
      double hgap = dist - 2.0 * rad;
      if (!(dist < dist0)) continue;
      double dist1 = 0.0;
      if (hgap < 0.0) dist1 = -hgap;
      double t = (dist0 - dist) / mingap;
      double fp = (t * t / pp.stf0 + dist1 / mingap / pp.stf1) * pp.fpc;
      double fpd = fp / dist;
      if (p == id) {
        acc[0] = acc[0] + fpd * dxij; acc[1] = acc[1] + fpd * dyij; acc[2] = acc[2] + fpd * dzij;
      } else {
        acc[0] = acc[0] - fpd * dxij; acc[1] = acc[1] - fpd * dyij; acc[2] = acc[2] - fpd * dzij;
      }
    }
  }
  if (lane != 0) return;
  if (channel) {
    // particle-wall lubrication, C/partlib.f90:2316-2355
    const double mw = pp.mingap_w;
    const double d0 = mw + rad;
    double xd = y[3 * p];
    double dist = xd, hgap = dist - rad;
    if (dist < d0) {
      double dist1 = hgap < 0.0 ? -hgap : 0.0;
      double t = (d0 - dist) / mw;
      double fp = (t * t / pp.stf0_w + dist1 / mw / pp.stf1_w) * pp.fpc;
      acc[0] = acc[0] + fp;
    }
    dist = (double)g.nx - xd;
    hgap = dist - rad;
    if (dist < d0) {
      double dist1 = hgap < 0.0 ? -hgap : 0.0;
      double t = (d0 - dist) / mw;
      double fp = (t * t / pp.stf0_w + dist1 / mw / pp.stf1_w) * pp.fpc;
      acc[0] = acc[0] - fp;
    }
  }
  ms.flubp[3 * p] = acc[0];
  ms.flubp[3 * p + 1] = acc[1];
  ms.flubp[3 * p + 2] = acc[2];
}
__global__ void k_lubforce(Geometry g, int npart, PartParams pp, MoveState ms) {
  k_lubforce_body(blockIdx.x, gridDim.x, g, npart, pp, ms);
}

// beads_move, B/partlib.f90:2305-2370, one thread per particle.  Also saves
// the pre-move centre (ypglbp, used by beads_filling).
__device__ __forceinline__ void move_particle(int p, int npart, PartParams pp, MoveState ms) {
  if (p >= npart) return;
  const bool first = *ms.first_move != 0;
  const double dt = 1.0;
  double fp[3], fpp[3], dwdtn[3], domgdtn[3];
  if (first) for (int c = 0; c < 3; ++c) ms.thetap[3 * p + c] = 0.0;
  for (int c = 0; c < 3; ++c) {
    ms.wpp[3 * p + c] = ms.wp[3 * p + c];
    ms.omgpp[3 * p + c] = ms.omgp[3 * p + c];
    ms.ypglbp[3 * p + c] = ms.ypglb[3 * p + c];
  }
  for (int c = 0; c < 3; ++c) fp[c] = ms.fHIp[3 * p + c] + ms.flubp[3 * p + c];
  fp[1] = fp[1] + pp.body_force_y;
  for (int c = 0; c < 3; ++c) fpp[c] = first ? fp[c] : ms.forcepp[3 * p + c];
  for (int c = 0; c < 3; ++c) dwdtn[c] = 0.5 * (fp[c] + fpp[c]) / pp.amp;
  for (int c = 0; c < 3; ++c) {
    double dw = first ? dwdtn[c] : ms.dwdt[3 * p + c];
    double wpp = ms.wpp[3 * p + c];
    double w = wpp + 0.5 * dt * (dw + dwdtn[c]);
    ms.wp[3 * p + c] = w;
    ms.ypglb[3 * p + c] = ms.ypglb[3 * p + c] + 0.5 * dt * (w + wpp);
  }
  for (int c = 0; c < 3; ++c) {
    double tq = ms.torqp[3 * p + c];
    double tpp = first ? tq : ms.torqpp[3 * p + c];
    domgdtn[c] = 0.5 * (tq + tpp) / pp.aip;
  }
  for (int c = 0; c < 3; ++c) {
    double dom = first ? domgdtn[c] : ms.domgdt[3 * p + c];
    double opp_ = ms.omgpp[3 * p + c];
    double o = opp_ + 0.5 * dt * (dom + domgdtn[c]);
    ms.omgp[3 * p + c] = o;
    ms.thetap[3 * p + c] = ms.thetap[3 * p + c] + 0.5 * dt * (o + opp_);
  }
  for (int c = 0; c < 3; ++c) {
    ms.dwdt[3 * p + c] = dwdtn[c];
    ms.domgdt[3 * p + c] = domgdtn[c];
    ms.forcep[3 * p + c] = fp[c];
    ms.forcepp[3 * p + c] = fp[c];
    ms.torqpp[3 * p + c] = ms.torqp[3 * p + c];
  }
}
__device__ __forceinline__ void k_move_body(int bx, int gx, int npart, PartParams pp, MoveState ms) {
  move_particle(bx * blockDim.x + threadIdx.x, npart, pp, ms);
}
__global__ void k_move(int npart, PartParams pp, MoveState ms) {
  k_move_body(blockIdx.x, gridDim.x, npart, pp, ms);
}

__global__ void k_clear_first(int* first_move) { *first_move = 0; }

// beads_redistribute's periodic wrap, B/partlib.f90:2600-2613
__device__ __forceinline__ void wrap_particle(int p, Geometry g, int npart, MoveState ms) {
  if (p >= npart) return;
  double* y = ms.ypglb + 3 * p;
  double xc = y[0], yc = y[1], zc = y[2];
  if (!g.channel) {
    if (xc >= (double)g.nx) y[0] = y[0] - (double)g.nx;
    if (xc < 0.0) y[0] = y[0] + (double)g.nx;
  }
  if (yc >= (double)g.ny) y[1] = y[1] - (double)g.ny;
  if (yc < 0.0) y[1] = y[1] + (double)g.ny;
  if (zc >= (double)g.nz) y[2] = y[2] - (double)g.nz;
  if (zc < 0.0) y[2] = y[2] + (double)g.nz;
}
__device__ __forceinline__ void k_wrap_body(int bx, int gx, Geometry g, int npart, MoveState ms) {
  wrap_particle(bx * blockDim.x + threadIdx.x, g, npart, ms);
}
__global__ void k_wrap(Geometry g, int npart, MoveState ms) {
  k_wrap_body(blockIdx.x, gridDim.x, g, npart, ms);
}
// beads_move, the wrap and the nearest-image sweeps of beads_links for
// kMoveSweepParts particles per block of 3 kMoveSweepParts threads: thread
// t < kMoveSweepParts moves and wraps particle kMoveSweepParts bx + t, then
// thread t sweeps axis t % 3 of particle kMoveSweepParts bx + t / 3 (the
// fused time step; the sweeps need only their own particle's new centre).
// Eight particles (one warp) per block spread the serial FP64 chains over as
// many SMs as there are blocks.
constexpr int kMoveSweepParts = 8;
constexpr int kMoveSweepThreads = 3 * kMoveSweepParts;
__global__ void __launch_bounds__(kMoveSweepThreads) k_move_wrap_sweeps(Geometry g, int npart, PartParams pp,
                                                                     MoveState ms, ParticleView pv,
                                                                     LinkSlab ls) {
  if (threadIdx.x < kMoveSweepParts) {
    const int p = blockIdx.x * kMoveSweepParts + threadIdx.x;
    move_particle(p, npart, pp, ms);
    wrap_particle(p, g, npart, ms);
  }
  __syncthreads();
  k_link_sweeps_body(blockIdx.x, gridDim.x, g, pv, ls);
}
// beads_move followed by beads_redistribute's wrap, each particle's thread
// wrapping the centre it has just moved
__global__ void k_move_wrap(Geometry g, int npart, PartParams pp, MoveState ms) {
  k_move_body(blockIdx.x, gridDim.x, npart, pp, ms);
  k_wrap_body(blockIdx.x, gridDim.x, g, npart, ms);
}

// ovlpchk after a move (hgap = dist - 2 rad < 0 aborts the reference,
// B/partlib.f90:2630-2646); here it raises LBM_ERR_OVERLAP.  One warp per
// particle, partners with a larger id.
__device__ __forceinline__ void k_overlap_body(int bx, int gx, Geometry g, int npart, PartParams pp, MoveState ms, DevStatus* st) {
  const int p = (bx * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (p >= npart) return;
  const bool channel = g.channel != 0;
  const double* y = ms.ypglb;
  const double xc = y[3 * p], yc = y[3 * p + 1], zc = y[3 * p + 2];
  const float lim = (float)(2.0 * pp.rad + 1.0);
  for (int q = p + 1 + lane; q < npart; q += 32) {
    if (!near_pair(g, y, p, q, lim)) continue;
    double xb = y[3 * q], yb = y[3 * q + 1], zb = y[3 * q + 2];
    if (!channel) xb = near_img(xb, xc, g.nx, g.nxh);
    yb = near_img(yb, yc, g.ny, g.nyh);
    zb = near_img(zb, zc, g.nz, g.nzh);
    double dist = sqrt((xc - xb) * (xc - xb) + (yc - yb) * (yc - yb) + (zc - zb) * (zc - zb));
    double hgap = dist - 2.0 * pp.rad;
    if (hgap < 0.0) raise_error(st, LBM_ERR_OVERLAP, p);
  }
}
__global__ void k_overlap(Geometry g, int npart, PartParams pp, MoveState ms, DevStatus* st,
                          int* clear_first) {
  // clear_first: beads_move's end of the first move, once every move has read it
  if (clear_first && blockIdx.x == 0 && threadIdx.x == 0) *clear_first = 0;
  k_overlap_body(blockIdx.x, gridDim.x, g, npart, pp, ms, st);
}

// beads_filling (B/partlib.f90:2846-3094), in two kernels.
// k_fill_detect: one block per particle scans the particle's previous
// bounding box for nodes it covered last step (isnodes0 == p) that are fluid
// now and appends them to an event list.
// k_fill_events: one warp per event refills the node.  A refill reads only
// nodes that are fluid in both steps and writes only its own node, so the
// events are independent and their order does not matter.
__device__ __forceinline__ void k_fill_detect_body(int bx, int gx, Geometry g, ParticleView pv, PartParams pp,
                                                    const double* __restrict__ ypglbp,
                                                    const int32_t* __restrict__ isnodes,
                                                    const int32_t* __restrict__ isnodes0,
                                                    FillList fl, DevStatus* st) {
  const int id = bx;
  if (id >= pv.npart) return;
  const bool channel = g.channel != 0;
  // bounding box of the nodes covered at the previous step (0-based node i
  // has centre i + 0.5), formed once by thread 0 (FP64 instructions cost a
  // warp the same whatever its active lanes)
  __shared__ int s_box[5];  // finite, r, bx0, by0, bz0
  if (threadIdx.x == 0) {
    const double cx0 = ypglbp[3 * id], cy0 = ypglbp[3 * id + 1], cz0 = ypglbp[3 * id + 2];
    s_box[0] = isfinite(cx0) && isfinite(cy0) && isfinite(cz0);
    if (s_box[0]) {
      const int r = (int)ceil(pp.rad) + 2;
      s_box[1] = r;
      s_box[2] = (int)floor(cx0 - 0.5) - r;
      s_box[3] = (int)floor(cy0 - 0.5) - r;
      s_box[4] = (int)floor(cz0 - 0.5) - r;
    }
  }
  __syncthreads();
  if (!s_box[0]) return;
  const int r = s_box[1], bx0 = s_box[2], by0 = s_box[3], bz0 = s_box[4];
  const int w = 2 * r + 2;
  const int wx = min(w, g.nx), wy = min(w, g.ny), wz = min(w, g.nz);
  // One thread per row of the box: the nodes solid last step and fluid now
  // are the set bits of (old mask & ~new mask), so a row costs one or two
  // 32-bit words of each mask; only those nodes' ids are read.
  const uint32_t* m0 = solid_mask(isnodes0, g);
  const uint32_t* m1 = solid_mask(isnodes, g);
  for (int rr = threadIdx.x; rr < wy * wz; rr += PB) {
    const int oy = rr % wy, oz = rr / wy;
    const int j = ((by0 + oy) % g.ny + g.ny) % g.ny, k = ((bz0 + oz) % g.nz + g.nz) % g.nz;
    const size_t rowbase = ((size_t)k * g.ny + j) * g.sw;
    // the box's x range as up to two segments [a, b) of [0, nx)
    int sa[2], sb[2], ns = 0;
    if (channel) {
      const int a = max(bx0, 0), b = min(bx0 + wx, g.nx);
      if (a < b) { sa[0] = a; sb[0] = b; ns = 1; }
    } else if (wx == g.nx) {
      sa[0] = 0; sb[0] = g.nx; ns = 1;
    } else {
      const int a = ((bx0 % g.nx) + g.nx) % g.nx;
      if (a + wx <= g.nx) { sa[0] = a; sb[0] = a + wx; ns = 1; }
      else { sa[0] = a; sb[0] = g.nx; sa[1] = 0; sb[1] = a + wx - g.nx; ns = 2; }
    }
    for (int sgm = 0; sgm < ns; ++sgm) {
      const int a = sa[sgm], b = sb[sgm];
      for (int wi = a >> 5; wi <= (b - 1) >> 5; ++wi) {
        uint32_t bits = m0[rowbase + wi] & ~m1[rowbase + wi];
        const int lo = max(a - 32 * wi, 0), hi = min(b - 32 * wi, 32);
        const uint32_t keep = (hi >= 32 ? 0xffffffffu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
        bits &= keep;
        while (bits) {
          const int i = 32 * wi + __ffs(bits) - 1;
          bits &= bits - 1;
          const int n = i + g.nx * (j + g.ny * k);
          if (isnodes0[n] != id) continue;
          const int e = atomicAdd(fl.count, 1);
          if (e < fl.cap) {
            fl.node[e] = n;
            fl.part[e] = id;
          } else {
            raise_error(st, LBM_ERR_CAPACITY, id);
          }
        }
      }
    }
  }
}
__global__ void __launch_bounds__(PB) k_fill_detect(Geometry g, ParticleView pv, PartParams pp,
                                                    const double* __restrict__ ypglbp,
                                                    const int32_t* __restrict__ isnodes,
                                                    const int32_t* __restrict__ isnodes0,
                                                    FillList fl, DevStatus* st) {
  k_fill_detect_body(blockIdx.x, gridDim.x, g, pv, pp, ypglbp, isnodes, isnodes0, fl, st);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Warp sums of four values, every lane getting all four, in six adds a lane
// instead of twenty: the first two butterfly levels halve the values a lane
// carries (lanes below 16 keep a and b, the others c and d; then bit 8 picks
// one of the two), the last three sum the one value left; a fixed order, so
// deterministic.  Lane 0, 8, 16, 24 end with the sum of a, b, c, d.
template <typename R>
__device__ __forceinline__ void warp_sum4(R& a, R& b, R& c, R& d) {
  const int lane = threadIdx.x & 31;
  const bool lo16 = lane < 16;
  R u = lo16 ? a : c, v = lo16 ? b : d;
  u += __shfl_xor_sync(0xffffffffu, lo16 ? c : a, 16);
  v += __shfl_xor_sync(0xffffffffu, lo16 ? d : b, 16);
  const bool lo8 = (lane & 8) == 0;
  R w = lo8 ? u : v;
  w += __shfl_xor_sync(0xffffffffu, lo8 ? v : u, 8);
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
  a = __shfl_sync(0xffffffffu, w, 0);
  b = __shfl_sync(0xffffffffu, w, 8);
  c = __shfl_sync(0xffffffffu, w, 16);
  d = __shfl_sync(0xffffffffu, w, 24);
}

// equilibrium of one population, feqpnt (B/partlib.f90:3222-3247)
// (the same expression with c . u from selected components and FMAs: values
// to rounding, fewer FP64 instructions)
template <typename R>
__device__ __forceinline__ R feq_q(int q, R u9, R v9, R w9, R rho9) {
  const R usqr = R(1.5) * fma_r(u9, u9, fma_r(v9, v9, w9 * w9));
  if (q == 0) return R(1.0 / 3.0) * (rho9 - usqr);
  const int cx = cix(q), cy = ciy(q), cz = ciz(q);
  const R G = (cx == 0 ? R(0) : flip_if(cx < 0, u9)) + (cy == 0 ? R(0) : flip_if(cy < 0, v9)) +
              (cz == 0 ? R(0) : flip_if(cz < 0, w9));
  const R wq = q <= 6 ? R(1.0 / 18.0) : R(1.0 / 36.0);
  return wq * (fma_r(R(4.5) * G, G, fma_r(R(3.0), G, rho9)) - usqr);
}

template <typename T>
__device__ __forceinline__ void k_fill_events_body(int bx, int gx, Geometry g, ParticleView pv, PartParams pp,
                                                     const double* __restrict__ ypglbp,
                                                     const double* __restrict__ wpp,
                                                     const double* __restrict__ omgpp,
                                                     const int32_t* __restrict__ isnodes,
                                                     const int32_t* __restrict__ isnodes0, T* f,
                                                     FillList fl, DevStatus* st) {
  using R = T;  // refill arithmetic in the population precision
  const int lane = threadIdx.x & 31;
  const int warp = (bx * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gx * blockDim.x) >> 5;
  const int nev = min(*fl.count, fl.cap);
  const bool channel = g.channel != 0;
  const double rad = pp.rad;
  for (int e = warp; e < nev; e += nwarps) {
    const int n = fl.node[e];
    const int id = fl.part[e];
    const int i = n % g.nx, jk = n / g.nx;
    const int j = jk % g.ny, k = jk / g.ny;
    // back-trace of the surface point and the lattice direction closest to
    // the surface normal (partlib.f90:2861-2925); centre offsets in FP64
    double xc = ypglbp[3 * id], yc = ypglbp[3 * id + 1], zc = ypglbp[3 * id + 2];
    const double xpnt = (double)(i + 1) - 0.5, ypnt = (double)(j + 1) - 0.5 + 0.0,
                 zpnt = (double)(k + 1) - 0.5 + 0.0;
    if (!channel) xc = near_img(xc, xpnt, g.nx, g.nxh);
    yc = near_img(yc, ypnt, g.ny, g.nyh);
    zc = near_img(zc, zpnt, g.nz, g.nzh);
    const R dx = R(xpnt - xc), dy = R(ypnt - yc), dz = R(zpnt - zc);
    const R w1 = R(-0.5 * (pv.wp[3 * id] + wpp[3 * id]));
    const R w2 = R(-0.5 * (pv.wp[3 * id + 1] + wpp[3 * id + 1]));
    const R w3 = R(-0.5 * (pv.wp[3 * id + 2] + wpp[3 * id + 2]));
    const R omg1 = R(-0.5 * (pv.omgp[3 * id] + omgpp[3 * id]));
    const R omg2 = R(-0.5 * (pv.omgp[3 * id + 1] + omgpp[3 * id + 1]));
    const R omg3 = R(-0.5 * (pv.omgp[3 * id + 2] + omgpp[3 * id + 2]));
    const R aa = w1 * w1 + w2 * w2 + w3 * w3;
    const R bb = dx * w1 + dy * w2 + dz * w3;
    const R cc = dx * dx + dy * dy + dz * dz - R(rad) * R(rad);
    const R inv_aa = R(1) / aa;  // one division for bb / aa and cc / aa
    const R ddt0 = bb * inv_aa;
    const R ddt1 = sqrt(ddt0 * ddt0 - cc * inv_aa);
    R ddt = -ddt0 + ddt1;
    if (ddt < R(0)) ddt = R(0);
    if (ddt > R(1)) ddt = R(1);
    const R xp1 = dx + w1 * ddt, yp1 = dy + w2 * ddt, zp1 = dz + w3 * ddt;  // relative to centre
    const R xx0 = xp1 + (omg2 * zp1 - omg3 * yp1) * ddt;
    const R yy0 = yp1 + (omg3 * xp1 - omg1 * zp1) * ddt;
    const R zz0 = zp1 + (omg1 * yp1 - omg2 * xp1) * ddt;
    const R sq2 = sqrt(R(2.0));
    R prod0 = R(-100.0);
    int ipmx = 0;
#pragma unroll
    for (int ipop = 1; ipop < NPOP; ++ipop) {
      // c . x0 with the zero terms left out (the same value, fewer FP64 ops)
      const int cx = cix(ipop), cy = ciy(ipop), cz = ciz(ipop);
      auto term = [](int c, R v) { return flip_if(c < 0, v); };
      R prod = cx ? term(cx, xx0) : R(0);
      if (cy) prod = cx ? prod + term(cy, yy0) : term(cy, yy0);
      if (cz) prod = (cx || cy) ? prod + term(cz, zz0) : term(cz, zz0);
      if (ipop <= 6) prod = prod * sq2;
      if (prod > prod0) { ipmx = ipop; prod0 = prod; }
    }
    // non-equilibrium part copied from the neighbour along ipmx if it is
    // fluid in both steps (partlib.f90:2963-2995); lane q holds population q
    const int q = lane < NPOP ? lane : 0;
    R fnew = R(0);
    {
      bool have = false;
      int m = 0;
      if (ipmx > 0) {
        int i2 = i + cix(ipmx);
        bool ok = true;
        if (channel) ok = i2 >= 0 && i2 < g.nx;
        else i2 = wrapi(i2, g.nx);
        if (ok) {
          const int j2 = wrapi(j + ciy(ipmx), g.ny), k2 = wrapi(k + ciz(ipmx), g.nz);
          m = i2 + g.nx * (j2 + g.ny * k2);
          have = isnodes[m] < 0 && isnodes0[m] < 0;
        }
      }
      if (have) {
        const R fq = lane < NPOP ? R(ld_pop(g, f, (long long)q * g.N + m)) : R(0);
        R rho9 = fq;
        R u9 = cix(q) == 0 ? R(0) : flip_if(cix(q) < 0, fq);
        R v9 = ciy(q) == 0 ? R(0) : flip_if(ciy(q) < 0, fq);
        R ww9 = ciz(q) == 0 ? R(0) : flip_if(ciz(q) < 0, fq);
        warp_sum4(rho9, u9, v9, ww9);
        fnew = fq - feq_q<R>(q, u9, v9, ww9, rho9);
      }
    }
    // local mean density of the neighbours fluid in both steps
    // (partlib.f90:3008-3065); lane d-1 handles neighbour d
    int cnt = 0;
    R rs = R(0);
    if (lane < 18) {
      const int d = lane + 1;
      int i2 = i + cix(d);
      bool ok = true;
      if (channel) ok = i2 >= 0 && i2 < g.nx;
      else i2 = wrapi(i2, g.nx);
      if (ok) {
        const int j2 = wrapi(j + ciy(d), g.ny), k2 = wrapi(k + ciz(d), g.nz);
        const int m = i2 + g.nx * (j2 + g.ny * k2);
        if (isnodes[m] < 0 && isnodes0[m] < 0) {
          cnt = 1;
#pragma unroll
          for (int ii = 0; ii < NPOP; ++ii) rs += R(ld_pop(g, f, (long long)ii * g.N + m));
        }
      }
    }
    const int nghb = warp_sum(cnt);
    const R rsum = warp_sum(rs);
    const R rho9 = nghb > 0 ? rsum / R(nghb) : (channel ? R(0) : R(pp.rho0));
    // equilibrium with the rigid-body velocity at the node
    const R wx = R(pv.wp[3 * id]), wy = R(pv.wp[3 * id + 1]), wz = R(pv.wp[3 * id + 2]);
    const R ox = R(pv.omgp[3 * id]), oy = R(pv.omgp[3 * id + 1]), oz = R(pv.omgp[3 * id + 2]);
    const R u9 = wx + oy * dz - oz * dy;
    const R v9 = wy + oz * dx - ox * dz;
    const R w9 = wz + ox * dy - oy * dx;
    if (lane < NPOP) st_pop(g, f, (long long)q * g.N + n, T(fnew + feq_q<R>(q, u9, v9, w9, rho9)), st, id);
  }
}
template <typename T>
__global__ void __launch_bounds__(128, 8) k_fill_events(Geometry g, ParticleView pv, PartParams pp,
                                                     const double* __restrict__ ypglbp,
                                                     const double* __restrict__ wpp,
                                                     const double* __restrict__ omgpp,
                                                     const int32_t* __restrict__ isnodes,
                                                     const int32_t* __restrict__ isnodes0, T* f,
                                                     FillList fl, DevStatus* st) {
  k_fill_events_body<T>(blockIdx.x, gridDim.x, g, pv, pp, ypglbp, wpp, omgpp, isnodes, isnodes0, f, fl, st);
}

}  // namespace

// SMs of the current device (queried once)
int sm_count() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
      sms = 1;
  }
  return sms;
}

void launch_links(const Geometry& g, const ParticleView& pv, int32_t* isnodes, LinkSlab ls,
                  DevStatus* st, int alpha_fp32, cudaStream_t s, bool sweeps_done) {
  if (pv.npart <= 0) return;
  if (!sweeps_done)
    { k_link_sweeps<<<(3 * pv.npart + kSmallBlock - 1) / kSmallBlock, kSmallBlock, 0, s>>>(g, pv, ls); count_launch(); }
  { k_links<<<pv.npart, PB, 0, s>>>(g, pv, isnodes, ls, st, alpha_fp32); count_launch(); }
}

template <typename T>
void launch_bounce_back(const Geometry& g, const ParticleView& pv, const T* f, int pushed,
                        const int32_t* isnodes, LinkSlab ls, double* fHIp, double* torqp,
                        cudaStream_t s) {
  if (pv.npart <= 0) return;
  { k_bounce<T><<<pv.npart, bounce_threads<T>(), 0, s>>>(g, pv, f, pushed, isnodes, ls, fHIp, torqp); count_launch(); }
}

template <typename T>
void launch_bounce_scatter(const Geometry& g, const ParticleView& pv, T* f, int pushed,
                           LinkSlab ls, cudaStream_t s, DevStatus* st) {
  if (pv.npart <= 0) return;
  // four blocks per SM, looping over particles: the stores run beside the
  // particle kernels of the critical path and leave half of every SM's
  // thread slots to them
  const int sms = sm_count();
  const int nblk = pv.npart < 4 * sms ? pv.npart : 4 * sms;
  { k_bounce_store<T><<<nblk, PB, 0, s>>>(g, pv, f, pushed, ls, st); count_launch(); }
}

void launch_lubforce(const Geometry& g, int npart, const PartParams& pp, MoveState ms,
                     cudaStream_t s) {
  if (npart <= 0) return;
  { k_lubforce<<<(npart * 32 + 127) / 128, 128, 0, s>>>(g, npart, pp, ms); count_launch(); }
}

void launch_move(const Geometry& g, int npart, const PartParams& pp, MoveState ms,
                 cudaStream_t s) {
  if (npart <= 0) return;
  { k_move<<<(npart + kSmallBlock - 1) / kSmallBlock, kSmallBlock, 0, s>>>(npart, pp, ms); count_launch(); }
  { k_clear_first<<<1, 1, 0, s>>>(ms.first_move); count_launch(); }
}

void launch_redistribute(const Geometry& g, int npart, const PartParams& pp, MoveState ms,
                         DevStatus* st, cudaStream_t s) {
  if (npart <= 0) return;
  { k_wrap<<<(npart + kSmallBlock - 1) / kSmallBlock, kSmallBlock, 0, s>>>(g, npart, ms); count_launch(); }
  { k_overlap<<<(npart * 32 + 127) / 128, 128, 0, s>>>(g, npart, pp, ms, st, nullptr); count_launch(); }
}

bool launch_move_redistribute(const Geometry& g, int npart, const PartParams& pp, MoveState ms,
                              DevStatus* st, cudaStream_t s, cudaStream_t aux, cudaEvent_t fork,
                              cudaEvent_t join, const ParticleView* pv, LinkSlab* ls) {
  if (npart <= 0) return false;
  if (pv && ls)
    { k_move_wrap_sweeps<<<(npart + kMoveSweepParts - 1) / kMoveSweepParts, kMoveSweepThreads, 0, s>>>(g, npart, pp, ms, *pv, *ls); count_launch(); }
  else
    { k_move_wrap<<<(npart + kSmallBlock - 1) / kSmallBlock, kSmallBlock, 0, s>>>(g, npart, pp, ms); count_launch(); }
  cudaStream_t so = s;
  if (aux) {
    cudaEventRecord(fork, s);
    cudaStreamWaitEvent(aux, fork, 0);
    so = aux;
  }
  { k_overlap<<<(npart * 32 + 127) / 128, 128, 0, so>>>(g, npart, pp, ms, st, ms.first_move); count_launch(); }
  if (aux) cudaEventRecord(join, aux);
  return aux != nullptr;
}

template <typename T>
void launch_filling(const Geometry& g, const ParticleView& pv, const PartParams& pp,
                    const double* ypglbp, const double* wpp, const double* omgpp,
                    const int32_t* isnodes, const int32_t* isnodes0, T* f, FillList fl,
                    DevStatus* st, cudaStream_t s) {
  if (pv.npart <= 0) return;
  cudaMemsetAsync(fl.count, 0, sizeof(int), s);
  { k_fill_detect<<<pv.npart, PB, 0, s>>>(g, pv, pp, ypglbp, isnodes, isnodes0, fl, st); count_launch(); }
  // eight blocks of four warps per SM: one refill event per warp for up to
  // 32 events an SM (the events' serial FP64 chains then run side by side)
  const int sms = sm_count();
  { k_fill_events<T><<<8 * sms, 128, 0, s>>>(g, pv, pp, ypglbp, wpp, omgpp, isnodes, isnodes0, f, fl, st); count_launch(); }
}

// ---- many boxes per launch ------------------------------------------------
namespace {

#define BOX_OR_RETURN(nblocks_expr)                  \
  const BoxParticles& B = boxes[blockIdx.y];         \
  const int nblk = (nblocks_expr);                   \
  if ((int)blockIdx.x >= nblk) return;

__global__ void __launch_bounds__(bounce_threads<float>(), 8) k_bounce_multi(const BoxParticles* boxes) {
  BOX_OR_RETURN(B.pv.npart)
  k_bounce_body<float, bounce_threads<float>()>(blockIdx.x, nblk, B.g, B.pv, B.f, 1, B.flags_cur, B.ls,
                                                B.ms.fHIp, B.ms.torqp);
}
__global__ void __launch_bounds__(PB) k_bounce_store_multi(const BoxParticles* boxes) {
  BOX_OR_RETURN(B.pv.npart)
  k_bounce_store_body<float>(blockIdx.x, nblk, B.g, B.pv, B.f, 1, B.ls);
}
__global__ void k_lubforce_multi(const BoxParticles* boxes) {
  BOX_OR_RETURN((B.pv.npart * 32 + 127) / 128)
  k_lubforce_body(blockIdx.x, nblk, B.g, B.pv.npart, B.pp, B.ms);
}
__global__ void k_move_wrap_multi(const BoxParticles* boxes) {
  BOX_OR_RETURN((B.pv.npart + kSmallBlock - 1) / kSmallBlock)
  k_move_body(blockIdx.x, nblk, B.pv.npart, B.pp, B.ms);
  k_wrap_body(blockIdx.x, nblk, B.g, B.pv.npart, B.ms);
}
__global__ void k_overlap_multi(const BoxParticles* boxes) {
  BOX_OR_RETURN((B.pv.npart * 32 + 127) / 128)
  // the end of the first move, once every move of this box has read it
  if (blockIdx.x == 0 && threadIdx.x == 0) *B.ms.first_move = 0;
  k_overlap_body(blockIdx.x, nblk, B.g, B.pv.npart, B.pp, B.ms, B.st);
}
// the new step's flags: every id -1, the solid mask clear; the refill list empty
__global__ void k_reset_multi(const BoxParticles* boxes) {
  const BoxParticles& B = boxes[blockIdx.y];
  if (B.pv.npart <= 0) return;
  const long long N = B.g.N;
  const long long words = (long long)B.g.ny * B.g.nz * B.g.sw;
  uint32_t* mask = reinterpret_cast<uint32_t*>(B.flags_next + N);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N + words; t += stride) {
    if (t < N) B.flags_next[t] = -1;
    else mask[t - N] = 0u;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *B.fl.count = 0;
}
__global__ void k_link_sweeps_multi(const BoxParticles* boxes) {
  BOX_OR_RETURN((3 * B.pv.npart + kSmallBlock - 1) / kSmallBlock)
  k_link_sweeps_body(blockIdx.x, nblk, B.g, B.pv, B.ls);
}
__global__ void __launch_bounds__(PB) k_links_multi(const BoxParticles* boxes) {
  BOX_OR_RETURN(B.pv.npart)
  k_links_body(blockIdx.x, nblk, B.g, B.pv, B.flags_next, B.ls, B.st, 1);
}
__global__ void __launch_bounds__(PB) k_fill_detect_multi(const BoxParticles* boxes) {
  BOX_OR_RETURN(B.pv.npart)
  k_fill_detect_body(blockIdx.x, nblk, B.g, B.pv, B.pp, B.ms.ypglbp, B.flags_next, B.flags_cur, B.fl,
                     B.st);
}
constexpr int kFillBlocks = 8;
__global__ void __launch_bounds__(128) k_fill_events_multi(const BoxParticles* boxes) {
  BOX_OR_RETURN(B.pv.npart > 0 ? kFillBlocks : 0)
  k_fill_events_body<float>(blockIdx.x, nblk, B.g, B.pv, B.pp, B.ms.ypglbp, B.ms.wpp, B.ms.omgpp,
                            B.flags_next, B.flags_cur, B.f, B.fl, B.st);
}
#undef BOX_OR_RETURN

}  // namespace

void launch_particle_step_multi(const BoxParticles* boxes, int nb, int max_npart,
                                long long max_reset, cudaStream_t s) {
  if (nb <= 0 || max_npart <= 0) return;
  auto grid = [&](long long blocks) { return dim3((unsigned)(blocks > 0 ? blocks : 1), nb); };
  k_bounce_multi<<<grid(max_npart), bounce_threads<float>(), 0, s>>>(boxes); count_launch();
  k_bounce_store_multi<<<grid(max_npart), PB, 0, s>>>(boxes); count_launch();
  k_lubforce_multi<<<grid((max_npart * 32 + 127) / 128), 128, 0, s>>>(boxes); count_launch();
  k_move_wrap_multi<<<grid((max_npart + kSmallBlock - 1) / kSmallBlock), kSmallBlock, 0, s>>>(boxes); count_launch();
  k_overlap_multi<<<grid((max_npart * 32 + 127) / 128), 128, 0, s>>>(boxes); count_launch();
  const long long rb = (max_reset + 256 * 8 - 1) / (256 * 8);
  k_reset_multi<<<grid(rb < 1024 ? rb : 1024), 256, 0, s>>>(boxes); count_launch();
  k_link_sweeps_multi<<<grid((3 * max_npart + kSmallBlock - 1) / kSmallBlock), kSmallBlock, 0, s>>>(boxes); count_launch();
  k_links_multi<<<grid(max_npart), PB, 0, s>>>(boxes); count_launch();
  k_fill_detect_multi<<<grid(max_npart), PB, 0, s>>>(boxes); count_launch();
  k_fill_events_multi<<<grid(kFillBlocks), 128, 0, s>>>(boxes); count_launch();
}

template void launch_bounce_back<double>(const Geometry&, const ParticleView&, const double*,
                                         int, const int32_t*, LinkSlab, double*, double*,
                                         cudaStream_t);
template void launch_bounce_back<float>(const Geometry&, const ParticleView&, const float*, int,
                                        const int32_t*, LinkSlab, double*, double*,
                                        cudaStream_t);
template void launch_bounce_scatter<double>(const Geometry&, const ParticleView&, double*, int,
                                            LinkSlab, cudaStream_t, DevStatus*);
template void launch_bounce_scatter<float>(const Geometry&, const ParticleView&, float*, int,
                                           LinkSlab, cudaStream_t, DevStatus*);
template void launch_filling<double>(const Geometry&, const ParticleView&, const PartParams&,
                                     const double*, const double*, const double*,
                                     const int32_t*, const int32_t*, double*, FillList,
                                     DevStatus*, cudaStream_t);
template void launch_filling<float>(const Geometry&, const ParticleView&, const PartParams&,
                                    const double*, const double*, const double*,
                                    const int32_t*, const int32_t*, float*, FillList,
                                    DevStatus*, cudaStream_t);

// initpartvel with trilinear (iflag = 1), 3DBox.../partlib.f90:177-263 and
// 320-831; the channel's (3DChannel.../partlib.f90:182-268, 325-836) has no
// x image.  One thread per centre and component.  The cell is formed as the
// reference forms it (1-based node i at i - 0.5, i = int(x + 0.5)); on one
// domain the halo planes trilinear reads are the periodic images, so the
// eight nodes wrap into 1..n along the open axes.  Weights and sum are
// rounded in the reference's order with no fused multiply-add: FP64 fields
// give the reference's wp bit for bit.  A centre whose cell leaves the grid
// (x + 0.5 outside [0, n + 1) along an open axis, where the reference reads
// outside its halo planes; x + 0.5 outside [1, nx) in a channel, where it
// reads outside ux) is reported in *bad and gets wp = 0.
template <typename T>
__global__ void k_initpartvel(Geometry g, const T* __restrict__ ux, const T* __restrict__ uy,
                              const T* __restrict__ uz, const double* __restrict__ y, int npart,
                              double* __restrict__ wp, int* __restrict__ bad) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * npart) return;
  const int ip = t / 3, d = t - 3 * ip;
  const double xc = y[3 * ip], yc = y[3 * ip + 1], zc = y[3 * ip + 2];
  const double sx = __dadd_rn(xc, 0.5), sy = __dadd_rn(yc, 0.5), sz = __dadd_rn(zc, 0.5);
  const bool ok = (g.channel ? (sx >= 1.0 && sx < g.nx) : (sx >= 0.0 && sx < g.nx + 1.0)) &&
                  sy >= 0.0 && sy < g.ny + 1.0 && sz >= 0.0 && sz < g.nz + 1.0;
  if (!ok) {
    wp[t] = 0.0;
    atomicMin(bad, ip);
    return;
  }
  int i = (int)sx, j = (int)sy, k = (int)sz;
  const double tx = __dsub_rn(sx, (double)i), ty = __dsub_rn(sy, (double)j),
               tz = __dsub_rn(sz, (double)k);
  const double tx0 = __dsub_rn(1.0, tx), ty0 = __dsub_rn(1.0, ty), tz0 = __dsub_rn(1.0, tz);
  int ip1 = i + 1, jp1 = j + 1, kp1 = k + 1;
  if (i == 0) i = g.nx;
  if (ip1 > g.nx) ip1 = 1;
  if (j == 0) j = g.ny;
  if (jp1 > g.ny) jp1 = 1;
  if (k == 0) k = g.nz;
  if (kp1 > g.nz) kp1 = 1;
  const T* u = d == 0 ? ux : (d == 1 ? uy : uz);
  auto at = [&](int a, int b, int c) {
    return (double)u[((long long)(c - 1) * g.ny + (b - 1)) * g.nx + (a - 1)];
  };
  auto w3 = [](double a, double b, double c, double v) {
    return __dmul_rn(__dmul_rn(__dmul_rn(a, b), c), v);
  };
  double v0 = w3(tx0, ty0, tz0, at(i, j, k));
  v0 = __dadd_rn(v0, w3(tx, ty0, tz0, at(ip1, j, k)));
  v0 = __dadd_rn(v0, w3(tx, ty, tz0, at(ip1, jp1, k)));
  v0 = __dadd_rn(v0, w3(tx0, ty, tz0, at(i, jp1, k)));
  v0 = __dadd_rn(v0, w3(tx0, ty0, tz, at(i, j, kp1)));
  v0 = __dadd_rn(v0, w3(tx, ty0, tz, at(ip1, j, kp1)));
  v0 = __dadd_rn(v0, w3(tx, ty, tz, at(ip1, jp1, kp1)));
  v0 = __dadd_rn(v0, w3(tx0, ty, tz, at(i, jp1, kp1)));
  wp[t] = v0;
}

template <typename T>
void launch_initpartvel(const Geometry& g, const T* ux, const T* uy, const T* uz,
                        const double* y, int npart, double* wp, int* bad, cudaStream_t s) {
  if (npart <= 0) return;
  const int n = 3 * npart;
  k_initpartvel<T><<<(n + 127) / 128, 128, 0, s>>>(g, ux, uy, uz, y, npart, wp, bad);
  count_launch();
}

template void launch_initpartvel<double>(const Geometry&, const double*, const double*,
                                         const double*, const double*, int, double*, int*,
                                         cudaStream_t);
template void launch_initpartvel<float>(const Geometry&, const float*, const float*,
                                        const float*, const double*, int, double*, int*,
                                        cudaStream_t);

}  // namespace lbm
