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

namespace lbm {

namespace {

constexpr int PB = 256;  // threads per particle block

__device__ __forceinline__ double near_img(double c, double p, int n, int nh) {
  if ((c - p) > (double)nh) c = c - (double)n;
  if ((c - p) < -(double)nh) c = c + (double)n;
  return c;
}
__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// The reference's beads_links keeps shifting the particle centre toward the
// current point and never resets it inside its loop nest
// (B/partlib.f90:961-982).  sweep_at returns the value of such a centre
// coordinate at point jq (1-based, points p_j = j - 0.5) of one sweep over
// j = 1..n that starts from value c, evaluating the same two conditional
// shifts at every point.  fl(c - p) is monotone in p, so the shift
// predicates are monotone and the points where a shift fires are found by
// bisection instead of visiting every point.
__device__ double sweep_at(double c, int jq, int n, int nh) {
  const double dn = (double)n, dnh = (double)nh;
  int j = 1;
  for (int guard = 0; guard < 16; ++guard) {
    double p = (double)j - 0.5;
    if ((c - p) > dnh) c = c - dn;
    if ((c - p) < -dnh) c = c + dn;
    if (j >= jq) return c;
    int jn = jq;
    double p1 = (double)(j + 1) - 0.5;
    if ((c - p1) > dnh) {
      jn = j + 1;
    } else {
      double pq = (double)jq - 0.5;
      if ((c - pq) < -dnh) {
        int lo = j + 1, hi = jq;
        while (lo < hi) {
          int mid = (lo + hi) >> 1;
          if ((c - ((double)mid - 0.5)) < -dnh) hi = mid; else lo = mid + 1;
        }
        jn = lo;
      }
    }
    j = jn;
  }
  return c;
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
constexpr int MAXROWS = 1024;

// beads_links for one particle per block.
__global__ void __launch_bounds__(PB) k_links(Geometry g, ParticleView pv, int32_t* isnodes,
                                              LinkSlab ls, DevStatus* st) {
  using Scan = cub::BlockScan<int, PB>;
  __shared__ typename Scan::TempStorage scan_tmp;
  __shared__ int plane_k[MAXPLANES];
  __shared__ double plane_z[MAXPLANES];
  __shared__ int nplanes;
  __shared__ int row_k[MAXROWS], row_j[MAXROWS];
  __shared__ double row_z[MAXROWS], row_y[MAXROWS];
  __shared__ int nrows;
  __shared__ int base;
  __shared__ int fixed_ok;

  const int p = blockIdx.x;
  if (p >= pv.npart) return;
  const double rad = pv.rad;
  const double radp2 = rad * 1.0 + 2.0;
  const double rad2 = (rad * 1.0) * (rad * 1.0);
  const bool channel = g.channel != 0;
  const double x0 = pv.ypglb[3 * p] * 1.0, y0 = pv.ypglb[3 * p + 1] * 1.0,
               z0 = pv.ypglb[3 * p + 2] * 1.0;
  const int tid = threadIdx.x;

  if (tid == 0) {
    nplanes = 0; nrows = 0; base = 0; fixed_ok = 1;
  }
  __syncthreads();

  // ---- planes: k with |zz0| <= radp2, zc from the k-sweep starting at z0
  Cands cz = make_cands(z0, g.nz, radp2, true);
  int tz = cz.total();
  for (int c0 = 0; c0 < tz; c0 += PB) {
    int t = c0 + tid;
    int k = -1;
    double zc = 0.0;
    bool take = false;
    if (t < tz) {
      k = cz.at(t);
      zc = sweep_at(z0, k, g.nz, g.nzh);
      double zpnt = (double)k - 0.5 + 0.0;
      double zz0 = zpnt - zc;
      take = fabs(zz0) <= radp2;
    }
    int pos, tot;
    Scan(scan_tmp).ExclusiveSum(take ? 1 : 0, pos, tot);
    __syncthreads();
    if (take && nplanes + pos < MAXPLANES) { plane_k[nplanes + pos] = k; plane_z[nplanes + pos] = zc; }
    __syncthreads();
    if (tid == 0) nplanes = min(nplanes + tot, MAXPLANES);
    __syncthreads();
  }

  // ---- rows: per plane, j with the y condition; the y-sweep of plane 0
  // starts at y0, every later plane at the sweep's fixed point Y1
  const double Y1 = sweep_at(y0, g.ny, g.ny, g.nyh);
  if (tid == 0 && sweep_at(Y1, g.ny, g.ny, g.nyh) != Y1) fixed_ok = 0;
  Cands cy = make_cands(y0, g.ny, radp2, true);
  int ty = cy.total();
  int tpairs = nplanes * ty;
  for (int c0 = 0; c0 < tpairs; c0 += PB) {
    int t = c0 + tid;
    bool take = false;
    int k = 0, j = 0;
    double zc = 0.0, yc = 0.0;
    if (t < tpairs) {
      int pi = t / ty;
      j = cy.at(t - pi * ty);
      k = plane_k[pi];
      zc = plane_z[pi];
      yc = sweep_at(pi == 0 ? y0 : Y1, j, g.ny, g.nyh);
      double zz0 = ((double)k - 0.5 + 0.0) - zc;
      double yy0 = ((double)j - 0.5 + 0.0) - yc;
      take = channel ? (sqrt(yy0 * yy0 + zz0 * zz0) <= radp2) : (fabs(yy0) <= radp2);
    }
    int pos, tot;
    Scan(scan_tmp).ExclusiveSum(take ? 1 : 0, pos, tot);
    __syncthreads();
    if (take && nrows + pos < MAXROWS) {
      row_k[nrows + pos] = k; row_j[nrows + pos] = j;
      row_z[nrows + pos] = zc; row_y[nrows + pos] = yc;
    }
    __syncthreads();
    if (tid == 0) nrows = min(nrows + tot, MAXROWS);
    __syncthreads();
  }

  // ---- nodes: per row, i candidates; box x-sweep: row 0 starts at x0,
  // later rows at the fixed point X1.  The channel never shifts x.
  const double X1 = channel ? x0 : sweep_at(x0, g.nx, g.nx, g.nxh);
  if (tid == 0 && !channel && sweep_at(X1, g.nx, g.nx, g.nxh) != X1) fixed_ok = 0;
  Cands cx = make_cands(x0, g.nx, radp2, !channel);
  int tx = cx.total();
  int tnodes = nrows * tx;
  int32_t* code = ls.code + (long long)p * ls.cap;
  double* alph = ls.alpha + (long long)p * ls.cap;
  for (int c0 = 0; c0 < tnodes; c0 += PB) {
    int t = c0 + tid;
    int nl = 0;
    int i = 0, j = 0, k = 0;
    double xx0 = 0, yy0 = 0, zz0 = 0, rr0 = 0, xc = 0, yc = 0, zc = 0;
    unsigned linkmask = 0;
    if (t < tnodes) {
      int r = t / tx;
      i = cx.at(t - r * tx);
      j = row_j[r]; k = row_k[r];
      zc = row_z[r]; yc = row_y[r];
      double xpnt = (double)i - 0.5;
      xc = channel ? x0 : sweep_at(r == 0 ? x0 : X1, i, g.nx, g.nxh);
      xx0 = xpnt - xc;
      yy0 = ((double)j - 0.5 + 0.0) - yc;
      zz0 = ((double)k - 0.5 + 0.0) - zc;
      bool inside;
      if (channel) {
        rr0 = xx0 * xx0 + yy0 * yy0 + zz0 * zz0;
        inside = sqrt(rr0) <= radp2;
      } else {
        inside = fabs(xx0) <= radp2;
        rr0 = xx0 * xx0 + yy0 * yy0 + zz0 * zz0;
      }
      if (inside) {
        double rr01 = rr0 - rad2;
        long long node = (long long)(i - 1) + (long long)g.nx * ((j - 1) + (long long)g.ny * (k - 1));
        if (rr01 <= 0.0) {
          atomicMax(&isnodes[node], p);
        } else {
#pragma unroll
          for (int ipop = 1; ipop < NPOP; ++ipop) {
            double xx1 = (double)(i + cix(ipop)) - 0.5 - xc;
            double yy1 = (double)(j + ciy(ipop)) - 0.5 - yc + 0.0;
            double zz1 = (double)(k + ciz(ipop)) - 0.5 - zc + 0.0;
            double rr1 = xx1 * xx1 + yy1 * yy1 + zz1 * zz1;
            if (rr1 - rad2 <= 0.0) linkmask |= 1u << ipop;
          }
          nl = __popc(linkmask);
        }
      }
    }
    int pos, tot;
    Scan(scan_tmp).ExclusiveSum(nl, pos, tot);
    __syncthreads();
    if (nl > 0) {
      long long node = (long long)(i - 1) + (long long)g.nx * ((j - 1) + (long long)g.ny * (k - 1));
      int w = base + pos;
      for (int ipop = 1; ipop < NPOP; ++ipop) {
        if (!(linkmask & (1u << ipop))) continue;
        double xx1 = (double)(i + cix(ipop)) - 0.5 - xc;
        double yy1 = (double)(j + ciy(ipop)) - 0.5 - yc + 0.0;
        double zz1 = (double)(k + ciz(ipop)) - 0.5 - zc + 0.0;
        double rr1 = xx1 * xx1 + yy1 * yy1 + zz1 * zz1;
        double rr11 = rr1 - rad2;
        double aa = rr0 + rr1 - 2.0 * (xx0 * xx1 + yy0 * yy1 + zz0 * zz1);
        double bb = xx1 * (xx0 - xx1) + yy1 * (yy0 - yy1) + zz1 * (zz0 - zz1);
        double cc = rr11;
        double alpha0 = bb / aa;
        double alpha1 = sqrt(alpha0 * alpha0 - cc / aa);
        double alpha = -alpha0 + alpha1;
        alpha = 1.0 - alpha;
        if (w < ls.cap) {
          code[w] = (int32_t)(node * 32 + ipop);
          alph[w] = alpha;
        }
        ++w;
      }
    }
    __syncthreads();
    if (tid == 0) base += tot;
    __syncthreads();
  }
  if (tid == 0) {
    ls.count[p] = min(base, ls.cap);
    if (base > ls.cap) raise_error(st, LBM_ERR_CAPACITY, p);
    if (nplanes >= MAXPLANES || nrows >= MAXROWS) raise_error(st, LBM_ERR_CAPACITY, p);
    if (!fixed_ok) raise_error(st, LBM_ERR_STATE, p);
  }
}

// post-collision population q at node (i, j, k) (0-based) in either layout.
// pushed: the fused kernel has already moved it to its streaming target
// (or bounced it back in place at a channel wall).
template <typename T>
__device__ __forceinline__ double read_post(const Geometry& g, const T* f, int pushed, int q, int i,
                                            int j, int k) {
  long long n = (long long)i + (long long)g.nx * (j + (long long)g.ny * k);
  if (!pushed) return (double)f[q * g.N + n];
  int it = i + cix(q);
  if (g.channel && (it < 0 || it >= g.nx)) return (double)f[ipopp(q) * g.N + n];
  it = wrapi(it, g.nx);
  int jt = wrapi(j + ciy(q), g.ny), kt = wrapi(k + ciz(q), g.nz);
  return (double)f[q * g.N + (long long)it + (long long)g.nx * (jt + (long long)g.ny * kt)];
}

// beads_collision for one particle per block: every link computes the
// bounced population f9 (stored per link) and its momentum exchange.
template <typename T>
__global__ void __launch_bounds__(PB) k_bounce(Geometry g, ParticleView pv, const T* f, int pushed,
                                               const int32_t* __restrict__ isnodes, LinkSlab ls,
                                               double* fHIp, double* torqp) {
  using Red = cub::BlockReduce<double, PB>;
  __shared__ typename Red::TempStorage red_tmp;
  const int p = blockIdx.x;
  if (p >= pv.npart) return;
  const int cnt = ls.count[p];
  const int32_t* code = ls.code + (long long)p * ls.cap;
  const double* alph = ls.alpha + (long long)p * ls.cap;
  double* f9s = ls.f9 + (long long)p * ls.cap;
  const double w1 = pv.wp[3 * p], w2 = pv.wp[3 * p + 1], w3 = pv.wp[3 * p + 2];
  const double omg1 = pv.omgp[3 * p], omg2 = pv.omgp[3 * p + 1], omg3 = pv.omgp[3 * p + 2];
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const bool channel = g.channel != 0;
  for (int l = threadIdx.x; l < cnt; l += PB) {
    int cd = code[l];
    int ipop = cd & 31;
    long long node = cd >> 5;
    int i = (int)(node % g.nx);
    long long r = node / g.nx;
    int j = (int)(r % g.ny), k = (int)(r / g.ny);
    double alpha = alph[l];
    int ipp = ipopp(ipop);
    double xpnt = (double)(i + 1) - 0.5, ypnt = (double)(j + 1) - 0.5, zpnt = (double)(k + 1) - 0.5;
    double xc = pv.ypglb[3 * p], yc = pv.ypglb[3 * p + 1], zc = pv.ypglb[3 * p + 2];
    if (!channel) xc = near_img(xc, xpnt, g.nx, g.nxh);
    yc = near_img(yc, ypnt, g.ny, g.nyh);
    zc = near_img(zc, zpnt, g.nz, g.nzh);
    int ix = cix(ipop), iy = ciy(ipop), iz = ciz(ipop);
    int im1 = i - ix, im2 = i - 2 * ix;
    int jm1 = wrapi(j - iy, g.ny), km1 = wrapi(k - iz, g.nz);
    int jm2 = wrapi(j - 2 * iy, g.ny), km2 = wrapi(k - 2 * iz, g.nz);
    bool out1 = false, out2 = false;
    if (channel) {
      out1 = im1 < 0 || im1 >= g.nx;
      out2 = im2 < 0 || im2 >= g.nx;
    } else {
      im1 = wrapi(im1, g.nx);
      im2 = wrapi(im2, g.nx);
    }
    double xx0 = xpnt + (double)ix * alpha - xc;
    double yy0 = ypnt + (double)iy * alpha - yc;
    double zz0 = zpnt + (double)iz * alpha - zc;
    double ff1 = read_post(g, f, pushed, ipop, i, j, k);
    double uwx = w1 + omg2 * zz0 - omg3 * yy0;
    double uwy = w2 + omg3 * xx0 - omg1 * zz0;
    double uwz = w3 + omg1 * yy0 - omg2 * xx0;
    double uwpro = uwx * (double)ix + uwy * (double)iy + uwz * (double)iz;
    const double wwp = ipop <= 6 ? 1.0 / 18.0 : 1.0 / 36.0;
    double f9;
    if (alpha <= 0.5) {
      int ibm1, ibm2;
      double ff2 = 0.0, ff3 = 0.0;
      if (out1) ibm1 = 2;
      else {
        long long m1 = (long long)im1 + (long long)g.nx * (jm1 + (long long)g.ny * km1);
        ibm1 = isnodes[m1] >= 0 ? 1 : -1;
        if (ibm1 < 0) ff2 = read_post(g, f, pushed, ipop, im1, jm1, km1);
      }
      if (out2) ibm2 = 2;
      else {
        long long m2 = (long long)im2 + (long long)g.nx * (jm2 + (long long)g.ny * km2);
        ibm2 = isnodes[m2] >= 0 ? 1 : -1;
        if (ibm1 < 0 && ibm2 < 0) ff3 = read_post(g, f, pushed, ipop, im2, jm2, km2);
      }
      if (ibm1 > 0) {
        f9 = ff1 - 6.0 * wwp * uwpro;
      } else if (ibm2 > 0) {
        f9 = 2.0 * alpha * (ff1 - ff2) + ff2 - 6.0 * wwp * uwpro;
      } else {
        double c1 = alpha * (1.0 + 2.0 * alpha);
        double c2 = 1.0 - 4.0 * alpha * alpha;
        double c3 = -alpha * (1.0 - 2.0 * alpha);
        f9 = c1 * ff1 + c2 * ff2 + c3 * ff3 - 6.0 * wwp * uwpro;
      }
    } else {
      double ff2 = read_post(g, f, pushed, ipp, i, j, k);
      int ibm1;
      double ff3 = 0.0;
      if (out1) ibm1 = 2;
      else {
        long long m1 = (long long)im1 + (long long)g.nx * (jm1 + (long long)g.ny * km1);
        ibm1 = isnodes[m1] >= 0 ? 1 : -1;
        if (ibm1 < 0) ff3 = read_post(g, f, pushed, ipp, im1, jm1, km1);
      }
      if (ibm1 > 0) {
        double c1 = 0.5 / alpha;
        double c2 = 1.0 - c1;
        f9 = c1 * ff1 + c2 * ff2 - 6.0 * wwp * c1 * uwpro;
      } else {
        double c1 = 1.0 / alpha / (2.0 * alpha + 1.0);
        double c2 = (2.0 * alpha - 1.0) / alpha;
        double c3 = 1.0 - c1 - c2;
        f9 = c1 * ff1 + c2 * ff2 + c3 * ff3 - 6.0 * wwp * c1 * uwpro;
      }
    }
    f9s[l] = f9;
    double dff = ff1 + f9;
    double dxmom = dff * (double)ix, dymom = dff * (double)iy, dzmom = dff * (double)iz;
    acc[0] += dxmom;
    acc[1] += dymom;
    acc[2] += dzmom;
    acc[3] = acc[3] + dzmom * yy0 - dymom * zz0;
    acc[4] = acc[4] + dxmom * zz0 - dzmom * xx0;
    acc[5] = acc[5] + dymom * xx0 - dxmom * yy0;
  }
  for (int c = 0; c < 6; ++c) {
    double s = Red(red_tmp).Sum(acc[c]);
    __syncthreads();
    if (threadIdx.x == 0) {
      if (c < 3) fHIp[3 * p + c] = s; else torqp[3 * p + c - 3] = s;
    }
  }
}

// the bounce-back stores of beads_collision: f(ipp, x + c) = f9
// (B/partlib.f90:1605-1621).  In the pushed layout that pre-streaming slot
// already sits at its streaming target, the fluid node x itself.
template <typename T>
__global__ void __launch_bounds__(PB) k_bounce_store(Geometry g, ParticleView pv, T* f, int pushed,
                                                     LinkSlab ls) {
  const int p = blockIdx.x;
  if (p >= pv.npart) return;
  const int cnt = ls.count[p];
  const int32_t* code = ls.code + (long long)p * ls.cap;
  const double* f9s = ls.f9 + (long long)p * ls.cap;
  for (int l = threadIdx.x; l < cnt; l += PB) {
    int cd = code[l];
    int ipop = cd & 31;
    long long node = cd >> 5;
    int ipp = ipopp(ipop);
    if (pushed) {
      int i = (int)(node % g.nx);
      int it = i + cix(ipop);
      if (g.channel && (it < 0 || it >= g.nx)) continue;
      f[ipp * g.N + node] = T(f9s[l]);
    } else {
      int i = (int)(node % g.nx);
      long long r = node / g.nx;
      int j = (int)(r % g.ny), k = (int)(r / g.ny);
      int it = i + cix(ipop);
      if (g.channel && (it < 0 || it >= g.nx)) continue;
      it = wrapi(it, g.nx);
      int jt = wrapi(j + ciy(ipop), g.ny), kt = wrapi(k + ciz(ipop), g.nz);
      f[ipp * g.N + (long long)it + (long long)g.nx * (jt + (long long)g.ny * kt)] = T(f9s[l]);
    }
  }
}

// beads_lubforce, one thread per particle.  Contributions to particle p are
// accumulated in ascending partner id, the order in which the reference's
// pair loop (id ascending, jj > id) reaches them.  Pairs farther apart than
// the lubrication range contribute exact zeros in the reference and are
// skipped after a single-precision range test with a wide margin.
__global__ void k_lubforce(Geometry g, int npart, PartParams pp, MoveState ms) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npart) return;
  const bool channel = g.channel != 0;
  const double rad = pp.rad, mingap = pp.mingap;
  const double dist0 = 2.0 * rad + mingap;
  const float lim = (float)(dist0 + 1.0);
  const double* y = ms.ypglb;
  double acc[3] = {0.0, 0.0, 0.0};
  const float fpx = (float)y[3 * p], fpy = (float)y[3 * p + 1], fpz = (float)y[3 * p + 2];
  for (int q = 0; q < npart; ++q) {
    if (q == p) continue;
    float dx = fabsf((float)y[3 * q] - fpx), dy = fabsf((float)y[3 * q + 1] - fpy),
          dz = fabsf((float)y[3 * q + 2] - fpz);
    if (!channel) dx = fminf(dx, (float)g.nx - dx);
    dy = fminf(dy, (float)g.ny - dy);
    dz = fminf(dz, (float)g.nz - dz);
    if (dx > lim || dy > lim || dz > lim || dx * dx + dy * dy + dz * dz > lim * lim) continue;
    // the pair as the reference evaluates it: centre "c" is the lower id
    int id = min(p, q), jj = max(p, q);
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

// beads_move, B/partlib.f90:2305-2370, one thread per particle.  Also saves
// the pre-move centre (ypglbp, used by beads_filling).
__global__ void k_move(int npart, PartParams pp, MoveState ms) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
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

__global__ void k_clear_first(int* first_move) { *first_move = 0; }

// beads_redistribute's periodic wrap, B/partlib.f90:2600-2613
__global__ void k_wrap(Geometry g, int npart, MoveState ms) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
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

// ovlpchk after a move (hgap = dist - 2 rad < 0 aborts the reference,
// B/partlib.f90:2630-2646); here it raises LBM_ERR_OVERLAP.
__global__ void k_overlap(Geometry g, int npart, PartParams pp, MoveState ms, DevStatus* st) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npart) return;
  const bool channel = g.channel != 0;
  const double* y = ms.ypglb;
  const double xc = y[3 * p], yc = y[3 * p + 1], zc = y[3 * p + 2];
  const float lim = (float)(2.0 * pp.rad + 1.0);
  for (int q = p + 1; q < npart; ++q) {
    float dx = fabsf((float)y[3 * q] - (float)xc), dy = fabsf((float)y[3 * q + 1] - (float)yc),
          dz = fabsf((float)y[3 * q + 2] - (float)zc);
    if (!channel) dx = fminf(dx, (float)g.nx - dx);
    dy = fminf(dy, (float)g.ny - dy);
    dz = fminf(dz, (float)g.nz - dz);
    if (dx > lim || dy > lim || dz > lim) continue;
    double xb = y[3 * q], yb = y[3 * q + 1], zb = y[3 * q + 2];
    if (!channel) xb = near_img(xb, xc, g.nx, g.nxh);
    yb = near_img(yb, yc, g.ny, g.nyh);
    zb = near_img(zb, zc, g.nz, g.nzh);
    double dist = sqrt((xc - xb) * (xc - xb) + (yc - yb) * (yc - yb) + (zc - zb) * (zc - zb));
    double hgap = dist - 2.0 * pp.rad;
    if (hgap < 0.0) { raise_error(st, LBM_ERR_OVERLAP, p); return; }
  }
}

// feqpnt, B/partlib.f90:3222-3247
__device__ void feqpnt(double u9, double v9, double w9, double rho9, double* feq9) {
  double usqr = u9 * u9 + v9 * v9 + w9 * w9;
  usqr = 1.5 * usqr;
  feq9[0] = (1.0 / 3.0) * (rho9 - usqr);
#pragma unroll
  for (int ip = 1; ip < NPOP; ++ip) {
    double G = cix(ip) * u9 + ciy(ip) * v9 + ciz(ip) * w9;
    double w = ip <= 6 ? 1.0 / 18.0 : 1.0 / 36.0;
    feq9[ip] = w * (rho9 + 3.0 * G + 4.5 * G * G - usqr);
  }
}

// beads_filling, one block per particle: scans the particle's previous
// bounding box for nodes it covered last step (isnodes0 == p) that are
// fluid now, and refills them (B/partlib.f90:2846-3094).  Reads only nodes
// that are fluid in both steps, writes only refilled nodes.
template <typename T>
__global__ void __launch_bounds__(PB) k_filling(Geometry g, ParticleView pv, PartParams pp,
                                                const double* __restrict__ ypglbp,
                                                const double* __restrict__ wpp,
                                                const double* __restrict__ omgpp,
                                                const int32_t* __restrict__ isnodes,
                                                const int32_t* __restrict__ isnodes0, T* f) {
  const int id = blockIdx.x;
  if (id >= pv.npart) return;
  const bool channel = g.channel != 0;
  const double rad = pp.rad;
  const double cx0 = ypglbp[3 * id], cy0 = ypglbp[3 * id + 1], cz0 = ypglbp[3 * id + 2];
  // bounding box of the nodes covered at the previous step (0-based node
  // i has centre i + 0.5)
  const int r = (int)ceil(rad) + 2;
  const int bx0 = (int)floor(cx0 - 0.5) - r, by0 = (int)floor(cy0 - 0.5) - r,
            bz0 = (int)floor(cz0 - 0.5) - r;
  const int w = 2 * r + 2;
  const int wx = min(w, g.nx), wy = min(w, g.ny), wz = min(w, g.nz);
  const long long total = (long long)wx * wy * wz;
  const double sq2 = sqrt(2.0);
  for (long long t = threadIdx.x; t < total; t += PB) {
    int ox = (int)(t % wx);
    long long rr = t / wx;
    int oy = (int)(rr % wy), oz = (int)(rr / wy);
    int i = bx0 + ox, j = by0 + oy, k = bz0 + oz;
    if (channel) {
      if (i < 0 || i >= g.nx) continue;
    } else {
      i = ((i % g.nx) + g.nx) % g.nx;
    }
    j = ((j % g.ny) + g.ny) % g.ny;
    k = ((k % g.nz) + g.nz) % g.nz;
    long long n = (long long)i + (long long)g.nx * (j + (long long)g.ny * k);
    if (!(isnodes0[n] == id && isnodes[n] < 0)) continue;
    double xc = cx0 * 1.0, yc = cy0 * 1.0, zc = cz0 * 1.0;
    double xpnt = (double)(i + 1) - 0.5, ypnt = (double)(j + 1) - 0.5 + 0.0, zpnt = (double)(k + 1) - 0.5 + 0.0;
    if (!channel) xc = near_img(xc, xpnt, g.nx, g.nxh);
    yc = near_img(yc, ypnt, g.ny, g.nyh);
    zc = near_img(zc, zpnt, g.nz, g.nzh);
    double w1 = -0.5 * (pv.wp[3 * id] * 1.0 + wpp[3 * id] * 1.0);
    double w2 = -0.5 * (pv.wp[3 * id + 1] * 1.0 + wpp[3 * id + 1] * 1.0);
    double w3 = -0.5 * (pv.wp[3 * id + 2] * 1.0 + wpp[3 * id + 2] * 1.0);
    double omg1 = -0.5 * (pv.omgp[3 * id] * 1.0 + omgpp[3 * id] * 1.0);
    double omg2 = -0.5 * (pv.omgp[3 * id + 1] * 1.0 + omgpp[3 * id + 1] * 1.0);
    double omg3 = -0.5 * (pv.omgp[3 * id + 2] * 1.0 + omgpp[3 * id + 2] * 1.0);
    double aa = w1 * w1 + w2 * w2 + w3 * w3;
    double bb = (xpnt - xc) * w1 + (ypnt - yc) * w2 + (zpnt - zc) * w3;
    double cc = (xpnt - xc) * (xpnt - xc) + (ypnt - yc) * (ypnt - yc) +
                (zpnt - zc) * (zpnt - zc) - (rad * 1.0) * (rad * 1.0);
    double ddt0 = bb / aa;
    double ddt1 = sqrt(ddt0 * ddt0 - cc / aa);
    double ddt = -ddt0 + ddt1;
    if (ddt < 0.0) ddt = 0.0;
    if (ddt > 1.0) ddt = 1.0;
    double xp1 = xpnt + w1 * ddt, yp1 = ypnt + w2 * ddt, zp1 = zpnt + w3 * ddt;
    double xp2 = xp1 + (omg2 * (zp1 - zc) - omg3 * (yp1 - yc)) * ddt;
    double yp2 = yp1 + (omg3 * (xp1 - xc) - omg1 * (zp1 - zc)) * ddt;
    double zp2 = zp1 + (omg1 * (yp1 - yc) - omg2 * (xp1 - xc)) * ddt;
    double xx0 = xp2 - xc, yy0 = yp2 - yc, zz0 = zp2 - zc;
    double prod0 = -100.0;
    int ipmx = 0;
    for (int ipop = 1; ipop < NPOP; ++ipop) {
      double prod = (double)cix(ipop) * xx0 + (double)ciy(ipop) * yy0 + (double)ciz(ipop) * zz0;
      if (ipop <= 6) prod = prod * sq2;
      if (prod > prod0) { ipmx = ipop; prod0 = prod; }
    }
    double fnew[NPOP], f9[NPOP], feq9[NPOP];
    bool have = false;
    if (ipmx > 0) {
      int i2 = i + cix(ipmx);
      bool ok = true;
      if (channel) ok = i2 >= 0 && i2 < g.nx;
      else i2 = wrapi(i2, g.nx);
      if (ok) {
        int j2 = wrapi(j + ciy(ipmx), g.ny), k2 = wrapi(k + ciz(ipmx), g.nz);
        long long m = (long long)i2 + (long long)g.nx * (j2 + (long long)g.ny * k2);
        if (isnodes[m] < 0 && isnodes0[m] < 0) {
          have = true;
          double rho9 = 0.0, u9 = 0.0, v9 = 0.0, ww9 = 0.0;
          for (int ip = 0; ip < NPOP; ++ip) f9[ip] = (double)f[ip * g.N + m];
          for (int ip = 0; ip < NPOP; ++ip) {
            rho9 = rho9 + f9[ip];
            u9 = u9 + (double)cix(ip) * f9[ip];
            v9 = v9 + (double)ciy(ip) * f9[ip];
            ww9 = ww9 + (double)ciz(ip) * f9[ip];
          }
          feqpnt(u9, v9, ww9, rho9, feq9);
          for (int ip = 0; ip < NPOP; ++ip) fnew[ip] = f9[ip] - feq9[ip];
        }
      }
    }
    if (!have)
      for (int ip = 0; ip < NPOP; ++ip) fnew[ip] = 0.0;
    int nghb = 0;
    double rho9 = 0.0;
    for (int ipop = 1; ipop < NPOP; ++ipop) {
      int i2 = i + cix(ipop);
      if (channel) { if (i2 < 0 || i2 >= g.nx) continue; }
      else i2 = wrapi(i2, g.nx);
      int j2 = wrapi(j + ciy(ipop), g.ny), k2 = wrapi(k + ciz(ipop), g.nz);
      long long m = (long long)i2 + (long long)g.nx * (j2 + (long long)g.ny * k2);
      if (isnodes[m] < 0 && isnodes0[m] < 0) {
        nghb = nghb + 1;
        for (int ii = 0; ii < NPOP; ++ii) rho9 = rho9 + (double)f[ii * g.N + m];
      }
    }
    if (nghb > 0) rho9 = rho9 / (double)nghb;
    else rho9 = channel ? 0.0 : pp.rho0;
    xx0 = xpnt - xc; yy0 = ypnt - yc; zz0 = zpnt - zc;
    w1 = pv.wp[3 * id]; w2 = pv.wp[3 * id + 1]; w3 = pv.wp[3 * id + 2];
    omg1 = pv.omgp[3 * id]; omg2 = pv.omgp[3 * id + 1]; omg3 = pv.omgp[3 * id + 2];
    double u9 = w1 + omg2 * zz0 - omg3 * yy0;
    double v9 = w2 + omg3 * xx0 - omg1 * zz0;
    double ww9 = w3 + omg1 * yy0 - omg2 * xx0;
    feqpnt(u9, v9, ww9, rho9, feq9);
    for (int ip = 0; ip < NPOP; ++ip) f[ip * g.N + n] = T(fnew[ip] + feq9[ip]);
  }
}

}  // namespace

void launch_links(const Geometry& g, const ParticleView& pv, int32_t* isnodes, LinkSlab ls,
                  DevStatus* st, cudaStream_t s) {
  if (pv.npart <= 0) return;
  k_links<<<pv.npart, PB, 0, s>>>(g, pv, isnodes, ls, st);
}

template <typename T>
void launch_bounce_back(const Geometry& g, const ParticleView& pv, const T* f, int pushed,
                        const int32_t* isnodes, LinkSlab ls, double* fHIp, double* torqp,
                        cudaStream_t s) {
  if (pv.npart <= 0) return;
  k_bounce<T><<<pv.npart, PB, 0, s>>>(g, pv, f, pushed, isnodes, ls, fHIp, torqp);
}

template <typename T>
void launch_bounce_scatter(const Geometry& g, const ParticleView& pv, T* f, int pushed,
                           LinkSlab ls, cudaStream_t s) {
  if (pv.npart <= 0) return;
  k_bounce_store<T><<<pv.npart, PB, 0, s>>>(g, pv, f, pushed, ls);
}

void launch_lubforce(const Geometry& g, int npart, const PartParams& pp, MoveState ms,
                     cudaStream_t s) {
  if (npart <= 0) return;
  k_lubforce<<<(npart + 127) / 128, 128, 0, s>>>(g, npart, pp, ms);
}

void launch_move(const Geometry& g, int npart, const PartParams& pp, MoveState ms,
                 cudaStream_t s) {
  if (npart <= 0) return;
  k_move<<<(npart + 127) / 128, 128, 0, s>>>(npart, pp, ms);
  k_clear_first<<<1, 1, 0, s>>>(ms.first_move);
}

void launch_redistribute(const Geometry& g, int npart, const PartParams& pp, MoveState ms,
                         DevStatus* st, cudaStream_t s) {
  if (npart <= 0) return;
  k_wrap<<<(npart + 127) / 128, 128, 0, s>>>(g, npart, ms);
  k_overlap<<<(npart + 127) / 128, 128, 0, s>>>(g, npart, pp, ms, st);
}

template <typename T>
void launch_filling(const Geometry& g, const ParticleView& pv, const PartParams& pp,
                    const double* ypglbp, const double* wpp, const double* omgpp,
                    const int32_t* isnodes, const int32_t* isnodes0, T* f, cudaStream_t s) {
  if (pv.npart <= 0) return;
  k_filling<T><<<pv.npart, PB, 0, s>>>(g, pv, pp, ypglbp, wpp, omgpp, isnodes, isnodes0, f);
}

template void launch_bounce_back<double>(const Geometry&, const ParticleView&, const double*,
                                         int, const int32_t*, LinkSlab, double*, double*,
                                         cudaStream_t);
template void launch_bounce_back<float>(const Geometry&, const ParticleView&, const float*, int,
                                        const int32_t*, LinkSlab, double*, double*,
                                        cudaStream_t);
template void launch_bounce_scatter<double>(const Geometry&, const ParticleView&, double*, int,
                                            LinkSlab, cudaStream_t);
template void launch_bounce_scatter<float>(const Geometry&, const ParticleView&, float*, int,
                                           LinkSlab, cudaStream_t);
template void launch_filling<double>(const Geometry&, const ParticleView&, const PartParams&,
                                     const double*, const double*, const double*,
                                     const int32_t*, const int32_t*, double*, cudaStream_t);
template void launch_filling<float>(const Geometry&, const ParticleView&, const PartParams&,
                                    const double*, const double*, const double*,
                                    const int32_t*, const int32_t*, float*, cudaStream_t);

}  // namespace lbm
