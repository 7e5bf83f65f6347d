/*
 * lbm.h - C ABI of the GB300 lattice Boltzmann engine (D3Q19 MRT with
 * finite-size moving spheres).
 *
 * The engine replaces the no-argument Fortran subroutines that the
 * reference main loop calls once per time step
 * (3DBox_Forced_HI_Turbulence_Moving_Particles_LBM/main.f90:172-188 and
 * 3DChannel_Decaying_HIT_Finite_Size_Moving_Particles/main.f90:187-204):
 *
 *   FORCING -> collision_MRT -> beads_collision -> streaming ->
 *   beads_lubforce -> beads_move -> beads_redistribute -> beads_links ->
 *   beads_filling -> macrovar
 *
 * The state that module var_inc shares between those subroutines
 * (3DBox.../var_inc.f90:70-103) lives on the GPU inside an lbm_ctx.  Every
 * entry point below takes plain host pointers and sizes; host arrays use the
 * reference's Fortran memory order, so a Fortran caller passes its own
 * arrays through ISO_C_BINDING without copying them first.
 *
 * Conventions shared by every entry point:
 *  - return 0 (LBM_OK) on success, a negative LBM_ERR_* code on failure;
 *    lbm_last_error() then describes the failure.  Nothing aborts the
 *    process (the reference's `stop` statements become error codes).
 *  - calls on one context are serialised on the context's CUDA stream and
 *    are not thread-safe; different contexts may be driven from different
 *    host threads.
 *  - no host pointer is retained after a call returns.
 *  - particle ids are 0-based here; the reference's ids are 1-based
 *    (isnodes = ip in 3DBox.../partlib.f90:992), so isnodes(i,j,k) = ip-1.
 */
#ifndef LBM_GB300_LBM_H
#define LBM_GB300_LBM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  LBM_OK = 0,
  LBM_ERR_ARG = -1,       /* bad argument or unsupported configuration       */
  LBM_ERR_CUDA = -2,      /* a CUDA runtime call failed                      */
  LBM_ERR_OVERLAP = -3,   /* particles overlap after a move (partlib.f90:2641) */
  LBM_ERR_CAPACITY = -4,  /* a fixed-capacity device list overflowed         */
  LBM_ERR_ALPHA = -5,     /* link fraction outside [0,1] (partlib.f90:1026):
                           * the reference prints and continues there, and so
                           * do the engine's link kernels; reserved          */
  LBM_ERR_NONFINITE = -6, /* non-finite value detected in the state          */
  LBM_ERR_TIMEOUT = -7,   /* a bounded device-side wait ran out              */
  LBM_ERR_STATE = -8,     /* call out of order (e.g. no particles uploaded)  */
  LBM_ERR_NOMEM = -9      /* device allocation failed                        */
};

/* ---- configuration ------------------------------------------------------ */
enum { LBM_PREC_F64 = 0, LBM_PREC_F32 = 1 };
/* LBM_BC_XWALLS: halfway bounce-back walls at x = 0 and x = nx, periodic in
 * y and z (3DChannel.../streaming.f90:11-13,175-187). */
enum { LBM_BC_PERIODIC = 0, LBM_BC_XWALLS = 1 };
/* LBM_FORCING_STOCHASTIC: low-wavenumber Ornstein-Uhlenbeck forcing
 * (3DBox.../gaussian.f90:182-372); LBM_FORCING_CONSTANT: uniform body force
 * (0, force_y, 0) (3DChannel.../collision.f90:335-347). */
enum { LBM_FORCING_NONE = 0, LBM_FORCING_STOCHASTIC = 1, LBM_FORCING_CONSTANT = 2 };
/* preset selector for lbm_config_init */
enum { LBM_PRESET_BOX = 0, LBM_PRESET_CHANNEL = 1 };

typedef struct lbm_config {
  int32_t nx, ny, nz;     /* lattice nodes per axis (lx = nx, ly = ny, lz = nz) */
  int32_t npart_max;      /* particle capacity (0: no particles)               */
  int32_t mrt_type;       /* 1, 2 or 3 as in para.f90:96-135                   */
  int32_t boundary;       /* LBM_BC_*                                          */
  int32_t forcing;        /* LBM_FORCING_*                                     */
  int32_t precision;      /* LBM_PREC_*                                        */
  int32_t iseedf;         /* forcing RNG seed, para.f90:20 (232300)           */
  int32_t iseedp;         /* particle position RNG seed, para.f90:247 (12345) */
  int32_t link_capacity;  /* links per particle (0: derived from rad)         */
  int32_t reserved_i[5];
  double visc;            /* kinematic viscosity; tau = 3 visc + 0.5          */
  double rho0;            /* reference density (1)                            */
  double rhopart;         /* particle density (var_inc.f90:27)                */
  double rad;             /* particle radius (var_inc.f90:28)                 */
  double mingap;          /* particle-particle lubrication range              */
  double mingap_w;        /* particle-wall lubrication range (channel)        */
  double vscale;          /* forcing velocity scale, para.f90:37              */
  double force_y;         /* constant body force per volume (channel)         */
  double fpc;             /* lubrication scale: volp*rho0*9.8/gscale (box,
                             partlib.f90:2260) or volp*rho0*g_lbm (channel)   */
  double stf0, stf1;      /* particle-particle stiffness, para.f90:244-245    */
  double stf0_w, stf1_w;  /* particle-wall stiffness (channel para.f90)       */
  double body_force_y;    /* extra y force added in beads_move:
                             -volp*rhog (box, partlib.f90:2332) or
                             +volp*force_in_y (channel partlib.f90:2409)     */
  double reserved_d[6];
} lbm_config;

/* Fill `cfg` with the reference's values for an n^3 box (para.f90) or an
 * nx*ny*nz x-walled channel (channel para.f90) holding `npart` spheres of
 * radius `rad` and density `rhopart`.  visc defaults to 0.0036. */
int lbm_config_init(lbm_config* cfg, int preset, int nx, int ny, int nz,
                    int npart, double rad, double rhopart);

/* ---- context ------------------------------------------------------------ */
typedef struct lbm_ctx lbm_ctx;

int lbm_create(const lbm_config* cfg, lbm_ctx** out);  /* allocates all device state */
/* The configuration a context was created with, and its particle count. */
int lbm_get_config(const lbm_ctx* ctx, lbm_config* cfg);
int lbm_particle_count(const lbm_ctx* ctx, int* npart);
int lbm_destroy(lbm_ctx* ctx);
const char* lbm_last_error(const lbm_ctx* ctx);         /* never NULL */
int lbm_version(void);                                  /* ABI version (1) */
/* bytes of device memory a context with this configuration allocates */
int lbm_footprint(const lbm_config* cfg, uint64_t* bytes);
/* Use `stream` (a cudaStream_t) for all work of this context; NULL = the
 * context's own stream. */
int lbm_set_stream(lbm_ctx* ctx, void* stream);
int lbm_synchronize(lbm_ctx* ctx);

/* ---- populations and macroscopic fields (var_inc.f90:89-92) ------------- */
/* f(0:18, lx, ly, lz) in Fortran order (population index fastest), FP64.
 * Replaces reading/writing var_inc's f. */
int lbm_upload_f(lbm_ctx* ctx, const double* f);
int lbm_download_f(lbm_ctx* ctx, double* f);
/* structure-of-arrays form f[q][z][y][x], q = 0..18, FP64 */
int lbm_upload_f_soa(lbm_ctx* ctx, const double* f);
int lbm_download_f_soa(lbm_ctx* ctx, double* f);
/* initpop (3DBox.../initial.f90:3-28): f = feq(rho' = 0, u) for a velocity
 * field given as three (lx, ly, lz) Fortran-order arrays. */
int lbm_initpop(lbm_ctx* ctx, const double* ux, const double* uy, const double* uz);
/* rho, ux, uy, uz as left by the last macrovar (each lx*ly*lz, Fortran order) */
int lbm_download_macro(lbm_ctx* ctx, double* rho, double* ux, double* uy, double* uz);
/* the body force field force_real{x,y,z} last produced by lbm_forcing */
int lbm_download_force(lbm_ctx* ctx, double* fx, double* fy, double* fz);

/* ---- particles (var_inc.f90:95-103) -------------------------------------- */
/* Release `npart` particles: ypglb, wp, omgp as (3, npart) Fortran arrays
 * (x,y,z fastest).  Equivalent to the `istep == irelease` block of
 * main.f90:149-165 with given positions and velocities; builds the links
 * (beads_links) and marks the next beads_move as the first one. */
int lbm_upload_particles(lbm_ctx* ctx, int npart, const double* ypglb,
                         const double* wp, const double* omgp);
/* initpartvel (3DBox.../partlib.f90:177-263 with trilinear, 320-831;
 * 3DChannel.../partlib.f90:182-268, 325-836): the fluid velocity at each of
 * `npart` centres ypglb (3, npart) by trilinear interpolation of the last
 * macrovar's u between the eight surrounding nodes, into wp (3, npart).
 * Periodic images along the open axes, as the reference's halo planes give
 * them; FP64 contexts reproduce the reference's rounding bit for bit.
 * LBM_ERR_ARG for a centre whose cell leaves the grid (x + 0.5 outside
 * [0, n + 1) along an open axis; in a channel, x + 0.5 outside [1, nx),
 * where the reference reads outside ux).  The context's particles are not
 * changed. */
int lbm_initpartvel(lbm_ctx* ctx, int npart, const double* ypglb, double* wp);
/* The release block of the reference's main loop (3DBox.../main.f90:149-165,
 * 3DChannel.../main.f90:163-175) with given centres: initpartvel, then
 * initpartomg, whose interpolated spin the reference discards (omgp = 0,
 * partlib.f90:927-929), then lbm_upload_particles (beads_links). */
int lbm_release_particles(lbm_ctx* ctx, int npart, const double* ypglb);
/* any pointer may be NULL; each is a (3, npart) array */
int lbm_download_particles(lbm_ctx* ctx, double* ypglb, double* wp, double* omgp,
                           double* fHIp, double* flubp, double* torqp);
/* The whole particle state, for checkpoints: dir 0 gets, dir 1 sets.
 * `state` holds 15 (3, npart) Fortran arrays back to back, in var_inc's
 * names (B/var_inc.f90:95-103): ypglb, ypglbp, wp, wpp, omgp, omgpp, dwdt,
 * domgdt, forcep, forcepp, torqp, torqpp, thetap, fHIp, flubp.  first_move
 * (may be NULL; 0 when NULL on set) is 1 when the next beads_move is the
 * first after release (partlib.f90:2310).  Setting rebuilds the solid flags
 * and links from ypglb (beads_links), as the reference's restart does after
 * loadcntdpart (main.f90:129-132).  npart must equal the context's on get. */
int lbm_particle_state(lbm_ctx* ctx, int dir, int npart, double* state, int32_t* first_move);
/* ibnodes (1 solid, -1 fluid) and isnodes (particle id, -1 fluid); each
 * lx*ly*lz int32 in Fortran order; either may be NULL */
int lbm_download_flags(lbm_ctx* ctx, int32_t* ibnodes, int32_t* isnodes);
/* The current boundary links (the nonzero entries of ilink/mlink/alink,
 * partlib.f90:1013-1024), grouped by particle and in (z, y, x, ipop) order
 * inside each particle.  node = i + lx*(j + ly*k) (0-based), ipop = 1..18.
 * Returns the link count in *nlinks; arrays may be NULL to query the count. */
int lbm_download_links(lbm_ctx* ctx, int64_t capacity, int64_t* nlinks,
                       int32_t* node, int32_t* ipop, int32_t* particle,
                       double* alpha);

/* ---- forcing state (gaussian.f90:182-215, saveload.f90:217-274) --------- */
/* dir = 0: read (iseedf, iyf, ivf[32], b[3*150]) from the context;
 * dir = 1: write them.  b holds b1r, b2r, b3r, each (6,5,5) Fortran order. */
int lbm_forcing_state(lbm_ctx* ctx, int dir, int32_t* iseedf, int32_t* iyf,
                      int32_t* ivf, double* b);

/* ---- the reference subroutines, one entry each --------------------------- */
int lbm_forcing(lbm_ctx* ctx);            /* gaussian.f90:182  FORCING        */
int lbm_collision_mrt(lbm_ctx* ctx);      /* collision.f90:8   collision_MRT  */
int lbm_beads_collision(lbm_ctx* ctx);    /* partlib.f90:1064  beads_collision*/
int lbm_streaming(lbm_ctx* ctx);          /* streaming.f90:2   streaming      */
int lbm_beads_lubforce(lbm_ctx* ctx);     /* partlib.f90:2211  beads_lubforce */
int lbm_beads_move(lbm_ctx* ctx);         /* partlib.f90:2295  beads_move     */
int lbm_beads_redistribute(lbm_ctx* ctx); /* partlib.f90:2397  (wrap+overlap) */
int lbm_beads_links(lbm_ctx* ctx);        /* partlib.f90:934   beads_links    */
int lbm_beads_filling(lbm_ctx* ctx);      /* partlib.f90:2793  beads_filling  */
int lbm_macrovar(lbm_ctx* ctx);           /* collision.f90:232 macrovar       */
int lbm_rhoupdat(lbm_ctx* ctx);           /* collision.f90:213 rhoupdat       */
/* The density pre-relaxation of a new run (B/main.f90:86-108, C/main.f90:
 * 71-95): repeat collision_MRT, streaming, rhoupdat with the velocity held
 * fixed until max|rho - rho_previous| <= eps or the iteration counter passes
 * max_iter (the reference: rhoepsl = 1e-5, 15000).  iters: the counter at
 * exit (the reference's printed istep); err: the last max difference.  One
 * 8-byte read-back per iteration. */
int lbm_prerelax(lbm_ctx* ctx, double eps, int max_iter, int* iters, double* err);

/* The whole time step of main.f90:172-188, `nsteps` times, fused into a
 * short chain of kernels per step.  Leaves the same state as calling the
 * entries above in that order. */
int lbm_step(lbm_ctx* ctx, int nsteps);

/* ---- initial conditions on the device (no counterpart in the reference) --- */
/* initpop (initial.f90:3-28) from a seeded divergence-free Gaussian velocity
 * field made on the GPU in the steps of initvel (initial.f90:55-116):
 * Gaussian modes projected off k, the kx = 0 plane Hermitian, the mean, the
 * Nyquist wavenumbers and the shells beyond nek = int(nx/2 - 1.5) zeroed,
 * each shell int(|k| + 1/2) = ik scaled to hold exactly ik^4 exp(-2 (ik/k0)^2)
 * (the workload's spectrum in place of initvel's), inverse FFT (cuFFT), and
 * one factor on all components so that sqrt(<|u|^2>/3) = u_rms.  initvel
 * draws from the Intel runtime's rand(), whose sequence is not published,
 * so the draws come from a counter-based generator instead.  Same seed,
 * same field. */
int lbm_init_spectral(lbm_ctx* ctx, double k0, double u_rms, uint64_t seed);
/* initpop from the channel's initial velocity, initvel of
 * 3DChannel.../initial.f90:57-126: the log-law mean flow in y between the
 * walls at x = 0 and x = nx (y+ ustar for y+ < 10.8, else
 * (ln(y+)/0.41 + 5) ustar; ustar = 360 visc / nx, ystar = visc / ustar),
 * u = w = 0 (the reference's perturbation amplitude is 0).  Needs a box
 * with walls (LBM_BC_XWALLS). */
int lbm_init_channel(lbm_ctx* ctx);
/* initpartpos (partlib.f90:1-80) with the ranpp generator and seed `seed`,
 * then lbm_upload_particles at rest.  LBM_ERR_OVERLAP if no placement is
 * found in max_rounds rounds (0: 100000). */
int lbm_init_particles(lbm_ctx* ctx, int npart, int seed, int max_rounds);
/* The placement of lbm_init_particles without a context or a GPU: initpartpos
 * (3DBox.../partlib.f90:1-80, 3DChannel.../partlib.f90:10-24) for the grid,
 * boundary, rad, mingap and mingap_w of cfg; centres into ypglb (3, npart),
 * the reference's var_inc layout.  LBM_ERR_OVERLAP if no placement is found in
 * max_rounds rounds (0: 100000).  Host code only: it may be called from any
 * thread while the GPU runs. */
int lbm_place_particles(const lbm_config* cfg, int npart, int seed, int max_rounds,
                        double* ypglb);
/* Deterministic summary of the current state: out[0] mass (sum f), out[1..3]
 * momentum, out[4] checksum sum_q,n (1 + q/19 + (n mod 97)/97) f, out[5]
 * kinetic energy sum (u.u)/2 of the last macrovar.  Bitwise equal for
 * bitwise equal states. */
int lbm_summary(lbm_ctx* ctx, double out[6]);

/* ---- statistics (saveload.f90:1111-1338) --------------------------------- */
/* Energy spectrum, dissipation and velocity-derivative moments of the
 * velocity left by the last macrovar, as statistc computes them: forward FFT
 * normalised by 1/N per axis, shells ik = int(|k| + 1/2), ik = 1..nshell,
 * nshell = int(nx/2 - 1.5), the kx = 0 plane weighted 1/2.
 *   ek[ik-1]  energy of shell ik (statistc's e_t, lattice units)
 *   dk[ik-1]  dissipation 2 nu |k|^2 E of shell ik with k = 2 pi (kx/nx,
 *             ky/ny, kz/nz) (statistc's e_ts times (2 pi / n)^2)
 *   out[0] nshell, out[1] kinetic energy sum ek, out[2] dissipation sum dk,
 *   out[3] skewness, out[4] flatness (statistc's formulas, which use wx in
 *   place of wz), out[5] u' = sqrt(2 out[1] / 3)
 * nek: length of ek and dk (entries past it are not written).  The first
 * call allocates FFT plans and work space (about 3 x 2 N doubles). */
int lbm_statistics(lbm_ctx* ctx, int nek, double* ek, double* dk, double* out);
/* Slip velocity of every particle, (3, npart) Fortran order: w_p minus the
 * mean fluid velocity over the fluid nodes at distance r_in <= r <= r_out
 * from the centre.  (Interpolating the velocity at the centre, as the
 * reference's trilinear does for initpartvel, returns the particle's own
 * rigid-body velocity once macrovar fills the solid nodes, so the slip is
 * taken on a fluid shell instead.)  No counterpart in the reference. */
int lbm_particle_slip(lbm_ctx* ctx, double r_in, double r_out, double* slip);
/* rmsstat (B/saveload.f90:1530-1730): the columns of rms.dat after the time,
 * out[36] = nf, nf/nx^3, mean u (3), rms u (3), velfrms, velfmn, mean wp (3),
 * rms wp (3), velprms, velpmn, mean vorticity (3), rms vorticity (3),
 * omgfrms/2, omgfmn, mean omgp (3), rms omgp (3), omgprms, omgpmn,
 * omgfrms^2, velfrms^2.  Fluid statistics over the nodes with isnodes < 0;
 * the vorticity is vortcalc's spectral curl with integer wavenumbers (the
 * Nyquist modes dropped); particle columns are 0 before release; omgpmn
 * takes the x mean twice as the reference does. */
int lbm_rmsstat(lbm_ctx* ctx, double* out);
/* diag (B/saveload.f90:1342-1400) without the time: out[5] = max |u| over
 * fluid nodes, idwp (1-based, first of equal maxima; 0 without particles),
 * max |wp|, idomgp, max |omgp|. */
int lbm_diag(lbm_ctx* ctx, double* out);
/* The channel's wall-normal profiles, statistc (fluid_only 0, 13 columns)
 * and statistc2 (fluid_only 1, 15 columns) of C/saveload.f90:1136-1428: per
 * x-plane i = 1..nx, out[(i-1)*ncol + c] = x = i - 1/2, y+, mean u, v, w /
 * ustar, their variances, the stresses uw, uv, vw, mean rho / ustar^2, its
 * variance, and (statistc2) the fluid and solid area fractions.  statistc
 * averages over the whole plane, statistc2 over its fluid nodes.  ustar <= 0:
 * from the channel force, force_y = 2 rho0 ustar^2 / nx (C/para.f90:15-17);
 * y+ uses ystar = visc / ustar. */
int lbm_channel_profiles(lbm_ctx* ctx, int fluid_only, double ustar, double* out);

/* ---- kernel selection (no counterpart in the reference) ------------------ */
/* Variants of the fused stream + collide kernel of lbm_step.  Both compute
 * the same per-node arithmetic; they differ in how the populations move. */
enum {
  LBM_VARIANT_DIRECT = 1, /* one thread per node: loads and pushed stores straight to HBM */
  LBM_VARIANT_STAGED = 2, /* persistent CTAs: a producer warp streams whole x-rows into
                             shared memory with bulk copies, consumer warps collide and
                             push them (nx a multiple of 4)                               */
  LBM_VARIANT_STAGED_X2 = 3 /* the same in FP32 with two nodes per thread on packed f32x2
                             arithmetic (FP32 precision, nx a multiple of 4, at most 512) */
};
/* Select a variant and its schedule.  For the staged variants: stages
 * (2..8: rows in flight + 1; 0: default), groups (STAGED_X2 only: groups of
 * consumer warps, each colliding its own row; 0: one) and ctas_per_sm (0: as
 * many as fit).  LBM_ERR_ARG when the variant or schedule does not apply to
 * this box.  A new context uses, where it applies, STAGED_X2 in FP32, else
 * STAGED in FP32, else DIRECT. */
int lbm_set_variant(lbm_ctx* ctx, int variant, int stages, int groups, int ctas_per_sm);
int lbm_get_variant(lbm_ctx* ctx, int* variant, int* stages, int* groups, int* ctas_per_sm);
/* Arithmetic of the collision in the fused stream + collide kernels.
 * LBM_SUMS_FLOAT: every operation in the populations' precision.
 * LBM_SUMS_FIXED (FP64 contexts): the sums with small integer coefficients
 * of the forward and inverse moment transforms are computed exactly in
 * 64-bit fixed point (2^-58 and 2^-61 resolution), and every product with a
 * rate, velocity or force stays FP64, so results agree with LBM_SUMS_FLOAT
 * to FP64 rounding.  A node whose populations or moments leave the fixed
 * point's range (|f| >= 1/8, scaled moments >= 1/32, not finite) or whose
 * populations are all below 2^-12 takes the FP64 path.  GB300 issues FP64 at
 * about 1/32 of its 32-bit integer rate, and these sums are most of the FP64
 * kernel's instructions.
 * LBM_SUMS_INTEGER (FP64 contexts, their default): LBM_SUMS_FIXED with the
 * velocity and force terms as exact 128-bit integer products of fixed-point
 * values too (products rounded once to 2^-64 or 2^-70, each term of a moment
 * once to 2^-61), so the collision issues no FP64 instruction on a node
 * that stays in range (|u| < 1/4, |F| < 2^-9; others take the FP64 path);
 * the body-force series is evaluated in FP64 beside it and rounded once to
 * its fixed point.
 * FP32 contexts accept LBM_SUMS_FLOAT only.  The unfused per-subroutine
 * entries always use LBM_SUMS_FLOAT.  No counterpart in the reference. */
enum { LBM_SUMS_FLOAT = 0, LBM_SUMS_FIXED = 1, LBM_SUMS_INTEGER = 2 };
int lbm_set_sums(lbm_ctx* ctx, int mode);
int lbm_get_sums(lbm_ctx* ctx, int* mode);
/* Time every applicable variant and schedule (reps launches each) on the
 * context's current populations without advancing them, keep the fastest and
 * report its mean milliseconds per launch.  Synchronises the stream. */
int lbm_autotune(lbm_ctx* ctx, int reps, double* best_ms);

/* ---- many boxes at once (no counterpart in the reference) ----------------- */
/* A batch advances several independent contexts together: each box's
 * FORCING and particle subroutines run on the box's own stream, and one
 * persistent kernel streams and collides every box.  Boxes must be FP32,
 * have nx a multiple of 4 and at most 128, share boundary, viscosity, MRT
 * rates and forcing kind, and be at the same step (all advanced equally
 * since creation).  A box gives the same result in a batch as alone through
 * a batch of one.  While batched, a context must not be stepped on its own;
 * reading its state (downloads, statistics) is allowed after
 * lbm_batch_synchronize.  lbm_batch_destroy returns the contexts to
 * standalone use. */
typedef struct lbm_batch lbm_batch;
int lbm_batch_create(lbm_ctx** ctxs, int n, lbm_batch** out);
int lbm_batch_destroy(lbm_batch* batch);
const char* lbm_batch_last_error(const lbm_batch* batch);
/* Advance every box nsteps steps.  use_graph = 1: whole cycles of 6 steps
 * (buffer parity x forcing-table rotation) are captured once into a CUDA
 * graph and replayed; the remainder runs directly.  Does not block. */
int lbm_batch_step(lbm_batch* batch, int nsteps, int use_graph);
/* Wait for the batch's work and report any device-side error of any box. */
int lbm_batch_synchronize(lbm_batch* batch);
/* Wait for the batch's work and report only the batched kernel's own
 * status; each box's errors are then read with lbm_synchronize(box). */
int lbm_batch_wait(lbm_batch* batch);
/* Schedule of the batched stream + collide kernel: stages (2..8), consumer
 * groups (1, 2 or 4; stages a multiple of groups), CTAs per SM (0: as many
 * as fit).  lbm_batch_autotune times every schedule on the current state
 * (without advancing it) and keeps the fastest. */
int lbm_batch_set_schedule(lbm_batch* batch, int stages, int groups, int ctas_per_sm);
int lbm_batch_get_schedule(lbm_batch* batch, int* stages, int* groups, int* ctas_per_sm);
int lbm_batch_autotune(lbm_batch* batch, int reps, double* best_ms);
/* total lattice nodes of the batch's boxes */
int64_t lbm_batch_nodes(const lbm_batch* batch);
/* Stream on which lbm_batch_step enqueues and finishes each call (the boxes'
 * own streams fork from and join back into it); NULL: the batch's own. */
int lbm_batch_set_stream(lbm_batch* batch, void* stream);

/* ---- serving (no counterpart in the reference) --------------------------- */
/* A request loop that keeps many solves resident on the GPU and advances
 * them together.  A request: grid (nx, ny, nz), wall_axis (-1: periodic box
 * with the stochastic forcing of the box preset; 0, 1, 2: halfway
 * bounce-back walls normal to x, y or z with the channel preset's constant
 * force), npart spheres of radius rad and density ratio rhopart placed by
 * initpartpos, precision, nsteps, and an initial field from
 * lbm_init_spectral(k0, u_rms, seed).  Requests are admitted in arrival
 * order (skipping ahead over requests that do not fit) while the sum of
 * lbm_footprint of the resident solves stays within hbm_budget bytes and at
 * most max_active are resident; FP32 boxes with constant forcing, wall-axis
 * extent a multiple of 4 and at most 128 are advanced by batches (one
 * persistent stream + collide kernel), the others on their own streams;
 * chunk_steps (even) bounds how many steps run between admissions.  A
 * request gives the same result alone and in any mix.  The loop runs on a
 * host thread of its own; submit, result, wait and stats may be called from
 * any thread. */
typedef struct lbm_server lbm_server;
typedef struct lbm_request {
  int32_t nx, ny, nz;
  int32_t wall_axis;
  int32_t npart;
  int32_t nsteps;
  int32_t precision;
  int32_t mrt_type;      /* 0: the preset's MRT rates; 1..3: MRTtype of para.f90 */
  int32_t keep_state;    /* 1: keep the finished solve's context for
                            lbm_server_take instead of destroying it       */
  int32_t reserved;
  double rad, rhopart;
  double k0, u_rms;
  uint64_t seed;
} lbm_request;
enum { LBM_REQ_QUEUED = 0, LBM_REQ_RUNNING = 1, LBM_REQ_DONE = 2, LBM_REQ_FAILED = 3 };
typedef struct lbm_result {
  int64_t id;
  int32_t state;       /* LBM_REQ_*                                             */
  int32_t error;       /* LBM_ERR_* when FAILED                                 */
  int32_t steps_done;
  int32_t batched;     /* 1 if some steps ran in a batch                        */
  double t_submit, t_start, t_done;  /* seconds since lbm_server_create       */
  double summary[6];   /* lbm_summary of the final state (momentum in the
                          request's axes)                                       */
} lbm_result;
int lbm_server_create(uint64_t hbm_budget, int max_active, int chunk_steps, lbm_server** out);
int lbm_server_submit(lbm_server* server, const lbm_request* req, int64_t* id);
int lbm_server_result(lbm_server* server, int64_t id, lbm_result* out);
/* block until request id is done or failed, at most timeout_s seconds
 * (LBM_ERR_TIMEOUT otherwise) */
int lbm_server_wait(lbm_server* server, int64_t id, double timeout_s);
/* out[13]: submitted, done, failed, resident, queued, HBM bytes in use,
 * batch regroupings, chunks advanced, seconds spent advancing, seconds since
 * creation, and the loop's seconds spent admitting (context set-up),
 * regrouping and retiring (summaries, context destruction) */
int lbm_server_stats(lbm_server* server, double* out);
/* The context of a finished request submitted with keep_state = 1: its
 * final populations, flags and particles, in the engine's axes (walls normal
 * to x; lbm_get_config gives the relabelled grid).  The caller owns it from
 * here and destroys it with lbm_destroy; until it is taken it stays resident
 * and counts against the server's HBM budget.  LBM_ERR_STATE if the request
 * is not done or kept nothing. */
int lbm_server_take(lbm_server* server, int64_t id, lbm_ctx** out);
/* stop the loop; resident solves end as LBM_REQ_FAILED (LBM_ERR_STATE);
 * kept contexts not taken are destroyed */
int lbm_server_destroy(lbm_server* server);

/* ---- diagnostics --------------------------------------------------------- */
/* FP64 totals over all nodes: out[0] = sum f (mass), out[1..3] = momentum
 * sum c f. */
int lbm_mass_momentum(lbm_ctx* ctx, double out[4]);

/* Device time per phase of the time step, from CUDA events recorded on the
 * context's stream around each phase.  enable = 1 clears the totals and
 * starts recording, 0 stops.  Phases (LBM_PHASE_*): */
enum {
  LBM_PHASE_STREAM_COLLIDE = 0, /* fused stream + MRT collide (or the unfused kernels) */
  LBM_PHASE_BOUNCE = 1,         /* beads_collision: bounce-back + stores              */
  LBM_PHASE_PARTICLES = 2,      /* beads_lubforce, beads_move, beads_redistribute     */
  LBM_PHASE_LINKS = 3,          /* beads_links (flag reset + link build)              */
  LBM_PHASE_FILLING = 4,        /* beads_filling                                      */
  LBM_PHASE_FORCING = 5,        /* FORCING (state update + force tables)              */
  LBM_NPHASES = 6
};
int lbm_profile(lbm_ctx* ctx, int enable);
/* total milliseconds and number of timed intervals of one phase since the
 * last lbm_profile(ctx, 1); synchronises the context's stream */
int lbm_profile_read(lbm_ctx* ctx, int phase, double* ms_total, int64_t* count);
/* number of kernels this library has launched in this process */
int64_t lbm_kernel_launches(void);
/* Measured FMA throughput (TFLOP/s, an FMA counted as 2 flops) of the
 * current device in FP64 (precision = LBM_PREC_F64) or FP32: the compute
 * roofline of the fused kernel.  No counterpart in the reference. */
int lbm_fma_throughput(int precision, double* tflops);

/* ---- allocation-free diagnostics ----------------------------------------- */
/* No counterpart in the reference.  Mass and momentum totals (out[0] = sum
 * f, out[1..3] = sum c f) of a population field the caller already holds on
 * the device, for callers that cannot allocate: a host solver that has
 * reserved the GPU's memory for its own state and forbids further
 * allocation, or an embedding runtime that owns all device memory through
 * its own pool.  Nothing is allocated (no cudaMalloc, cudaFree or allocating
 * library call; no context needed).
 *   f       device pointer, 19*nx*ny*nz doubles laid out f[q][z][y][x]
 *   out     device pointer to 4 doubles
 *   stream  cudaStream_t to run on (NULL: the legacy default stream); the
 *           call returns after enqueueing, out is ready when the stream is
 * Scratch is one file-scope 256-byte-aligned device array of
 * LBM_NOALLOC_MAX_PLANES x 4 doubles (128 KiB) that every GPU loading this
 * library holds until the process exits; nz > LBM_NOALLOC_MAX_PLANES is
 * rejected with LBM_ERR_ARG.  All calls share that array and it keeps the
 * last call's partial sums: calls that overlap on one GPU (for example on
 * two streams) race on it, so the caller must order them.  No entry needs
 * clearing between calls (each call writes every entry it reads).  Every
 * call looks up the array's device address in the current context (so a
 * caller's own driver-API context, or one recreated after cudaDeviceReset,
 * gets its own instance); the first call in a context also loads the
 * library's device code there, so make that first call before any stream
 * capture.  Returns LBM_ERR_STATE without launching anything when a CUDA
 * error is already pending from earlier work (left pending for its owner),
 * and LBM_ERR_CUDA when one of this call's own launches fails. */
#define LBM_NOALLOC_MAX_PLANES 4096
int lbm_mass_momentum_noalloc(const double* f, int nx, int ny, int nz, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_LBM_H */
