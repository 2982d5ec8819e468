/*
 * aeros_gpu.h -- C-ABI of the GB300 (sm_103a) spectral dynamics path.
 *
 * This is the drop-in boundary for aeros' spectral transform module and its
 * dry time step.  A Fortran host binds it with iso_c_binding through bind(C)
 * interfaces of these prototypes; Python binds it with ctypes
 * (aeros_gb300/_capi.py).
 *
 * Conventions (identical to the reference arrays, so a Fortran caller passes
 * its arrays straight through):
 *   - spectral arrays are complex(c_double) (nlm[, nbatch]), stored as
 *     interleaved (re, im) doubles, m-major: 0-based lm = m(2T+1-m)/2 + l
 *     (src/aeros_spectral.f90:478);
 *   - grid arrays are real(c_double) (nlon, nlat[, nbatch]), longitude
 *     contiguous, latitude north -> south (src/aeros_defs.f90:196-204);
 *   - orthonormal harmonics without the Condon-Shortley phase,
 *     Y_lm = Pbar_lm(cos theta) e^{i m phi} / sqrt(2 pi)
 *     (src/aeros_spectral.f90:17-27).
 * Pointers may be host or device memory; host buffers are staged through the
 * handle's device workspace, device buffers are used in place.
 *
 * Every entry point returns an int status: 0 = success, negative = error
 * (see AEROS_ERR_*).  Nothing aborts the process; the reference's
 * `stop 1` / `error stop 1` conditions come back as these codes.
 * A handle is not thread-safe and owns one CUDA stream.
 */
#ifndef AEROS_GPU_H
#define AEROS_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define AEROS_OK                 0
#define AEROS_ERR_ARG           -1   /* bad argument / shape              */
#define AEROS_ERR_CUDA          -2   /* CUDA runtime failure              */
#define AEROS_ERR_NOMEM         -3   /* device allocation failed          */
#define AEROS_ERR_SINGULAR      -4   /* singular Helmholtz matrix         */
#define AEROS_ERR_NONFINITE     -5   /* NaN/Inf detected in the state     */
#define AEROS_ERR_STATE         -6   /* call out of order                 */
#define AEROS_ERR_UNSUPPORTED   -7   /* size or mode not built            */

/* ---- precision modes of the Legendre contraction ------------------------ */
#define AEROS_PREC_FP64   0   /* plain FP64 (DFMA)                          */
#define AEROS_PREC_SPLIT  1   /* split-precision tensor-core (Ozaki) form   */

/* ---- opaque handles ------------------------------------------------------ */
typedef struct aeros_sht_s *aeros_sht_t;
typedef struct aeros_dyn_s *aeros_dyn_t;
typedef struct aeros_group_s *aeros_group_t;

/* ======================================================================== */
/* Spectral transforms: mirrors module aeros_spectral                        */
/* (src/aeros_spectral.f90:128-143)                                          */
/* ======================================================================== */

/* Smallest quadratically-unaliased Gaussian grid for truncation T:
 * nlon = 3T+1 rounded up to an even 2/3/5-smooth number, nlat = nlon/2.
 * Replaces aeros_sht_grid_size (src/aeros_spectral.f90:399-436). */
int aeros_sht_grid_size(int trunc, int *nlon, int *nlat);

/* Create a transform for truncation T on an (nlon, nlat) Gaussian grid
 * (nlon/nlat <= 0 pick the default grid) able to process up to `batch_max`
 * fields per call.  Replaces aeros_sht_init (src/aeros_spectral.f90:147-279)
 * and the per-thread pool aeros_sht_pool_init (:305-342): one handle per
 * stream replaces one SHTns config per OpenMP thread. */
int aeros_sht_create(aeros_sht_t *h, int trunc, int nlon, int nlat, int batch_max);

/* Release a transform.  Replaces aeros_sht_end (src/aeros_spectral.f90:281-303). */
int aeros_sht_destroy(aeros_sht_t h);

/* Realized configuration and geometry (host arrays; any pointer may be NULL):
 * sinlat (nlat) = Gauss nodes cos(colatitude) north->south, gauss_w (nlat)
 * summing to 2, l_of_lm / m_of_lm (nlm).  Replaces the geometry fields of
 * aeros_sht_class (src/aeros_spectral.f90:47-85). */
int aeros_sht_info(aeros_sht_t h, int *trunc, int *nlon, int *nlat, int *nlm,
                   double *sinlat, double *gauss_w, int *l_of_lm, int *m_of_lm);

/* 1-based index of (l, m), or -1 outside the truncation.
 * Replaces aeros_sht_lm (src/aeros_spectral.f90:460-482). */
int aeros_sht_lm(aeros_sht_t h, int l, int m);

/* Select the Legendre contraction precision (AEROS_PREC_*). */
int aeros_sht_set_precision(aeros_sht_t h, int mode);

/* Bind the handle to a caller's CUDA stream (cudaStream_t); NULL = own. */
int aeros_sht_set_stream(aeros_sht_t h, void *stream);

/* Scalar synthesis: coeffs (nlm, nbatch) -> field (nlon, nlat, nbatch).
 * Replaces aeros_sht_synthesis / SH_to_spat (src/aeros_spectral.f90:502-515). */
int aeros_sht_synthesis(aeros_sht_t h, const double *coeffs, double *field, int nbatch);

/* Scalar analysis: field (nlon, nlat, nbatch) -> coeffs (nlm, nbatch).  The
 * input is NOT destroyed (the reference's contract allows destruction, so this
 * is a superset).  Replaces aeros_sht_analysis / spat_to_SH (:486-500). */
int aeros_sht_analysis(aeros_sht_t h, const double *field, double *coeffs, int nbatch);

/* Vector synthesis: spheroidal/toroidal (slm, tlm) -> (v_theta, v_phi), unit
 * sphere, v_theta positive southward.  Replaces aeros_sht_synthesis_vec /
 * SHsphtor_to_spat (src/aeros_spectral.f90:545-558). */
int aeros_sht_synthesis_vec(aeros_sht_t h, const double *slm, const double *tlm,
                            double *vth, double *vph, int nbatch);

/* Vector analysis: (v_theta, v_phi) -> (slm, tlm); l = 0 returns zero.
 * Replaces aeros_sht_analysis_vec / spat_to_SHsphtor (:529-543). */
int aeros_sht_analysis_vec(aeros_sht_t h, const double *vth, const double *vph,
                           double *slm, double *tlm, int nbatch);

/* Gradient on the unit sphere: gth = dF/dtheta, gph = (1/sin theta) dF/dphi.
 * Replaces aeros_sht_gradient / SHsph_to_spat (src/aeros_spectral.f90:560-584). */
int aeros_sht_gradient(aeros_sht_t h, const double *coeffs, double *gth, double *gph,
                       int nbatch);

/* In-place Laplacian, x (-l(l+1)/a^2); inverse != 0 divides and zeroes l = 0.
 * Replaces aeros_sht_laplacian (src/aeros_spectral.f90:588-630). */
int aeros_sht_laplacian(aeros_sht_t h, double *coeffs, int inverse, int nbatch);

/* Global integral a^2 sum_j w_j (sum_i f_ij) 2pi/nlon for each of nbatch
 * fields, in FP64.  Replaces aeros_sht_surface_integral (:632-666). */
int aeros_sht_surface_integral(aeros_sht_t h, const double *field, double *total,
                               int nbatch);

/* Wind <-> vorticity/divergence, one call for nbatch levels, with the
 * reference's sign conventions (u = V_phi, v = -V_theta, S = -a D/(l(l+1)),
 * T = a zeta/(l(l+1)), l = 0 discarded).  Replace aeros_uv_from_vordiv,
 * aeros_vordiv_from_uv and aeros_gradient (src/dynamics/aeros_vordiv.f90:82-205). */
int aeros_uv_from_vordiv(aeros_sht_t h, const double *vor, const double *div,
                         double *u, double *v, int nbatch);
int aeros_vordiv_from_uv(aeros_sht_t h, const double *u, const double *v,
                         double *vor, double *div, int nbatch);
int aeros_gradient(aeros_sht_t h, const double *f, double *dfdx, double *dfdy, int nbatch);

/* Number of this library's kernel launches issued by the handle so far. */
int aeros_sht_launch_count(aeros_sht_t h, long long *count);

/* Scalar synthesis that allocates nothing, for callers that cannot call
 * cudaMalloc (device memory owned by another allocator or reserved up front,
 * or a loop whose memory must not change once it runs).  No counterpart in
 * the reference.  It always computes in FP64 (the handle's precision mode is
 * not used): on an FP64 handle the result is aeros_sht_synthesis's.  coeffs
 * and field must be device pointers, and the handle's device (the one current
 * at aeros_sht_create) must be the current device, else AEROS_ERR_ARG.  Its
 * Fourier-row scratch (2^19 complex = 8 MiB) and descriptors live in static
 * device arrays that every GPU loading the library holds until exit:
 * nbatch <= 256 and nlat * nbatch * (T+1) <= 2^19, else AEROS_ERR_ARG.  All
 * calls share those arrays, so calls that overlap on the GPU race.  The first
 * call on a device resolves the arrays' addresses.  Synchronous (it waits for
 * its stream), so it cannot be called inside a stream capture. */
int aeros_sht_synthesis_noalloc(aeros_sht_t h, const double *coeffs, double *field, int nbatch);

/* ======================================================================== */
/* Dry dynamics step: mirrors aeros_timestep / aeros facade                  */
/* ======================================================================== */

/* Configuration.  Field meanings follow aeros_param_class
 * (src/aeros_defs.f90:114-190), the &aeros_vert group
 * (src/dynamics/aeros_vertical.f90:95-124) and the Held-Suarez constants
 * (src/physics/aeros_held_suarez.f90:92-101), which are runtime values here so
 * that ensemble members can carry perturbed forcing. */
typedef struct aeros_params {
    int    trunc;          /* triangular truncation T                        */
    int    nlon, nlat;     /* <= 0: default grid for T                       */
    int    nlev;           /* full levels                                    */
    int    nmember;        /* ensemble members stepped together (>= 1)       */
    int    precision;      /* AEROS_PREC_*                                   */
    double dt;             /* time step [s]                                  */
    double eps_filter;     /* RAW filter nu                                  */
    double raw_alpha;      /* Williams alpha (1 = Robert-Asselin)            */
    double si_alpha;       /* semi-implicit decentering weight in [0.5, 1]   */
    double tau_diff;       /* diffusion e-folding at l = lmax [hours]        */
    int    ndiff;          /* diffusion order (even)                         */
    int    semi_implicit;  /* 0 = explicit leapfrog                          */
    int    held_suarez;    /* Held-Suarez forcing on/off                     */
    int    mass_fixer;     /* global mass fixer on/off                       */
    /* vertical grid generator */
    double stretch_a, stretch_r, sigma_t, p_top, ps_ref, t_ref;
    /* Held-Suarez constants */
    double hs_t_equator, hs_t_min, hs_dt_y, hs_dtheta_z, hs_sigma_b, hs_p0;
    double hs_k_a, hs_k_s, hs_k_f;   /* [s-1] */
} aeros_params;

/* Fill `p` with the Held-Suarez benchmark configuration of
 * par/held_suarez.nml (T31 L20, dt 1800 s, RAW 0.06/0.53, del^6 6 h, pure
 * sigma on [0.01, 1], t_ref 300 K, mass fixer on). */
int aeros_params_default(aeros_params *p);

/* Build the integrator: vertical grid, semi-implicit operators, diffusion
 * ratios, Held-Suarez factors, device state for p->nmember members.
 * a_half/b_half (nlev+1) may be NULL (generated from the stretching
 * parameters) or an explicit hybrid table; 2 to 64 levels (AEROS_ERR_UNSUPPORTED
 * above).  Replaces aeros_timestep_init
 * (src/dynamics/aeros_timestep.f90:452-598), aeros_vgrid_init
 * (src/dynamics/aeros_vertical.f90:126-298) and aeros_semiimp_init
 * (src/dynamics/aeros_semiimp.f90:171-276). */
int aeros_dyn_create(aeros_dyn_t *h, const aeros_params *p,
                     const double *a_half, const double *b_half);
int aeros_dyn_destroy(aeros_dyn_t h);

/* Geometry and vertical coordinate (host arrays, any may be NULL):
 * A, B (nlev+1), sigma_full (nlev), sinlat, gauss_w (nlat). */
int aeros_dyn_info(aeros_dyn_t h, int *nlon, int *nlat, int *nlm, int *nlev,
                   double *a_half, double *b_half, double *sigma_full,
                   double *sinlat, double *gauss_w);

/* Per-member Held-Suarez equator-pole contrast dT_y [K] and k_a [s-1]. */
int aeros_dyn_set_member_forcing(aeros_dyn_t h, int member, double dt_y, double k_a);

/* Install the spectral state X^n of every member and restart the leapfrog
 * (the next step is the start-up step).  vor/div/temp are (nlm, nlev,
 * nmember), lnps (nlm, nmember).  Mirrors writing ams%now%spec and
 * ts%nstep = 0 (src/aeros.f90:130-183). */
int aeros_dyn_set_state(aeros_dyn_t h, const double *vor, const double *div,
                        const double *temp, const double *lnps);
int aeros_dyn_get_state(aeros_dyn_t h, double *vor, double *div, double *temp,
                        double *lnps);
/* X^(n-1), for restarts (src/dynamics/aeros_timestep.f90:1303-1633). */
int aeros_dyn_set_old_state(aeros_dyn_t h, const double *vor, const double *div,
                            const double *temp, const double *lnps, int nstep);
int aeros_dyn_get_old_state(aeros_dyn_t h, double *vor, double *div, double *temp,
                            double *lnps);

/* Resting isothermal state at temp [K] and ps [Pa] (<= 0: reference values),
 * for all members.  Replaces aeros_set_isothermal (src/aeros.f90:130-183). */
int aeros_dyn_set_isothermal(aeros_dyn_t h, double temp, double ps);

/* Deterministic temperature seed of every member's current state: T_lm,k +=
 * amp (cos(3l + 5m + k), sin(7l + 2m + 3k)) for m = 1..8, l = m..m+4, k = 1..nlev.
 * Replaces aeros_hs_perturb (src/physics/aeros_held_suarez.f90:295-336). */
int aeros_dyn_hs_perturb(aeros_dyn_t h, double amp);

/* Surface geopotential (nlon, nlat) [m2 s-2], shared by all members.
 * Replaces aeros_timestep_set_phis (src/dynamics/aeros_timestep.f90:1817-1844). */
int aeros_dyn_set_phis(aeros_dyn_t h, const double *phis);

/* Advance every member by nsteps dynamics steps.  Replaces nsteps calls of
 * aeros_timestep_step (src/dynamics/aeros_timestep.f90:776-1137), dry path. */
int aeros_dyn_step(aeros_dyn_t h, int nsteps);

/* Facade clock (src/aeros.f90:60-124,202-241).  aeros_dyn_set_time sets the
 * model time at initialisation [yr] (aeros_init's optional time_init; 0 at
 * creation) and clears the facade's step count.  aeros_dyn_update advances to
 * `time` [yr] with the reference's rule: target = nint((time - time_init) *
 * year_seconds / dt) (halves rounded away from zero, year_seconds = 365.25 d),
 * take target - nstep steps when positive, then nstep = max(target, nstep) and
 * the clock reads `time`.  A time earlier than the clock is AEROS_ERR_ARG
 * ("cannot step backwards", the reference's stop 1) and steps nothing.  Grid
 * fields are read with aeros_dyn_diagnose, which always sees the current
 * state.  aeros_dyn_get_time returns the clock and the facade's step count. */
int aeros_dyn_set_time(aeros_dyn_t h, double time_init);
int aeros_dyn_update(aeros_dyn_t h, double time);
int aeros_dyn_get_time(aeros_dyn_t h, double *time, int *nstep);

/* Enqueue nsteps steps on the handle's stream and return at once (CUDA
 * graphs; no host synchronization).  aeros_dyn_sync waits for them and
 * reports AEROS_ERR_NONFINITE if any step produced a NaN/Inf. */
int aeros_dyn_step_async(aeros_dyn_t h, int nsteps);
/* A caller that keeps the state on the host, in one call: X^n (now_in) and
 * X^(n-1) (old_in) with its step count nstep in, nsteps steps, the new X^n
 * (now_out) and the new X^(n-1) (old_out: the RAW-filtered previous level,
 * which the next call takes as old_in) out; either output may be NULL.  Each
 * array is one time level packed vor | div | temp | lnps (all members each,
 * aeros_dyn_state_size complex values), host or device: the same as
 * aeros_dyn_set_state + aeros_dyn_set_old_state + aeros_dyn_step +
 * aeros_dyn_get_state + aeros_dyn_get_old_state with four copies and one
 * synchronisation.  With nsteps = 1 and every array device memory or pinned
 * host memory (aeros_host_register), the copies, the step and the error-word
 * reads are one CUDA graph launch, built for the call's pointers and reused
 * while they stay the same. */
int aeros_dyn_step_packed(aeros_dyn_t h, const double *now_in, const double *old_in, int nstep, int nsteps,
                          double *now_out, double *old_out);
/* Page-lock (cudaHostRegister) or release a host array so that copies from and
 * to it run at full speed and aeros_dyn_step_packed takes its one-graph form;
 * for a Fortran host's state arrays. */
int aeros_host_register(void *ptr, size_t bytes);
int aeros_host_unregister(void *ptr);
int aeros_dyn_sync(aeros_dyn_t h);

/* Run one step with a CUDA event after every kernel (no graph) and return the
 * per-kernel durations in ms (up to maxk) and their names (name_len bytes
 * each, may be NULL).  For measurement; the step is a real step. */
int aeros_dyn_profile_step(aeros_dyn_t h, int maxk, double *ms, char *names, int name_len, int *nk);

/* Adiabatic spectral tendencies R(X^n) of the current state, no forcing:
 * replaces aeros_tendency_calc (src/dynamics/aeros_tendency.f90:338-360). */
int aeros_dyn_tendency(aeros_dyn_t h, double *dvor, double *ddiv, double *dtemp,
                       double *dlnps);

/* Spectral tendencies with the forcing the step applies: Held-Suarez (when
 * enabled) and the physics hook (aeros_dyn_set_physics), both added on the
 * grid at the seam of aeros_tendency_grid / aeros_tendency_spectral
 * (src/dynamics/aeros_tendency.f90:362-388).  Same layout as
 * aeros_dyn_tendency. */
int aeros_dyn_tendency_forced(aeros_dyn_t h, double *dvor, double *ddiv, double *dtemp,
                              double *dlnps);

/* ---- tracer transport -----------------------------------------------------
 * Positive-definite finite-volume transport of a grid tracer
 * (src/dynamics/aeros_transport.f90): the tracer mass q dp and the layer air
 * mass dp advanced by the same van Leer (horizontal) and donor-cell or van Leer
 * (vertical) face fluxes, sub-stepped so the largest total Courant number is
 * at most 0.9.  Grids are (nlon, nlat, nlev) Fortran arrays, latitude north to
 * south; pointers host or device. */
typedef struct aeros_transport_s *aeros_transport_t;

/* aeros_transport_init (:155-203): Gaussian grid of truncation trunc, nlev
 * layers with half-level coefficients p_half = a_half + b_half ps (nlev + 1,
 * top to bottom, host memory; nlev <= 64). */
int aeros_transport_create(aeros_transport_t *h, int trunc, int nlev, const double *a_half,
                           const double *b_half);
int aeros_transport_destroy(aeros_transport_t h);
int aeros_transport_set_stream(aeros_transport_t h, void *stream);   /* NULL: the legacy default stream */
int aeros_transport_grid(aeros_transport_t h, int *nlon, int *nlat, int *nlev);
/* The vert_vanleer switch of aeros_transport_class (default off: donor cell). */
int aeros_transport_set_vert_vanleer(aeros_transport_t h, int on);
/* aeros_transport_transport (:225-287): advance q in place over dt [s] with the
 * winds u, v [m/s] and ln ps [ln Pa] (nlon, nlat). */
int aeros_transport_step(aeros_transport_t h, const double *u, const double *v, const double *lnps,
                         double *q, double dt);
/* last_cfl and last_nsub of the previous call. */
int aeros_transport_last(aeros_transport_t h, double *cfl, int *nsub);
/* aeros_transport_water (:743-779): total tracer mass [kg] of q with surface
 * pressure ps [Pa] (nlon, nlat). */
int aeros_transport_water(aeros_transport_t h, const double *ps, const double *q, double *water);

/* ---- physics seam ---------------------------------------------------------
 * The grid-space view a physics hook receives at the seam of
 * src/dynamics/aeros_tendency.f90:362-388: after the adiabatic right-hand
 * sides (and Held-Suarez forcing, when enabled) are formed on the grid and
 * before they are transformed back to spectral space, so a hook's
 * contribution is carried by the same transforms (and a horizontally varying
 * drag stays exact under the curl).  Device pointers to member 0, level 0;
 * field f of member e at level k starts at f + e * member_stride +
 * k * level_stride, each level an (nlon, nlat) grid, longitude fastest,
 * latitude north to south. */
typedef struct aeros_grid_view {
    int nmember, nlev, nlat, nlon;
    long long level_stride;        /* doubles between levels (nlat * nlon) */
    long long in_member_stride;    /* doubles between members of u .. lnps */
    long long out_member_stride;   /* doubles between members of ae .. dlnpsdt */
    const double *u, *v, *vor, *div, *temp, *lnps;   /* state on the grid (lnps: one level) */
    double *ae, *an, *dtdt, *dlnpsdt;                /* right-hand sides: add tendencies here */
    const double *sinlat;          /* (nlat), device */
    const double *a_half, *b_half; /* (nlev + 1) half-level coefficients, host memory */
    double dt;                     /* model time step [s] */
} aeros_grid_view;

/* A physics hook enqueues device work on `stream` (a cudaStream_t) that reads
 * the view's state and adds to its right-hand sides.  It is called on the
 * host whenever the handle enqueues its tendency work: when the step graphs
 * are captured (aeros_dyn_set_physics, aeros_dyn_autotune) and on every direct
 * launch (aeros_dyn_profile_step, aeros_dyn_tendency_forced); the captured
 * work is replayed every step.  It must only enqueue stream-ordered work (no
 * synchronisation, no allocation while capturing) and returns 0, or nonzero
 * to fail the call that invoked it.  The adjoint entry points refuse a handle
 * with a hook (they do not differentiate user physics). */
typedef int (*aeros_physics_fn)(void *user, const aeros_grid_view *view, void *stream);

/* Install (fn != NULL) or remove (fn == NULL) the hook and re-capture the step
 * graphs.  `user` is passed through unchanged and must outlive the hook.  An
 * ensemble group copies its members' step graphs when it is created: install
 * hooks before grouping. */
int aeros_dyn_set_physics(aeros_dyn_t h, aeros_physics_fn fn, void *user);

/* A ready-made hook, also the template for user physics: linear relaxation
 * with `user` pointing to an aeros_relaxation (host memory, read when the hook
 * runs):  ae -= k_drag u,  an -= k_drag v,  dtdt -= k_temp (T - t_ref). */
typedef struct aeros_relaxation {
    double k_drag;   /* [1/s] */
    double k_temp;   /* [1/s] */
    double t_ref;    /* [K] */
} aeros_relaxation;
int aeros_physics_relaxation(void *user, const aeros_grid_view *view, void *stream);

/* Grid-space fields of the current state: u, v, temp (nlon, nlat, nlev,
 * nmember), ps (nlon, nlat, nmember).  Replaces aeros_timestep_diagnose
 * (src/dynamics/aeros_timestep.f90:1873-1919). */
int aeros_dyn_diagnose(aeros_dyn_t h, double *u, double *v, double *temp, double *ps);

/* FP64 global mass [kg], total energy [J], angular momentum [kg m2 s-1] of
 * every member (nmember each).  Replaces aeros_budget_calc
 * (src/aeros_budget.f90:61-142). */
int aeros_dyn_budget(aeros_dyn_t h, double *mass, double *energy, double *angmom);

/* Mass fixer bookkeeping: steps taken, target mass, last and cumulative log
 * corrections of member 0 (src/dynamics/aeros_timestep.f90:1225-1301). */
int aeros_dyn_counters(aeros_dyn_t h, int *nstep, double *mass_target,
                       double *lnr_last, double *lnr_cum);
/* Set every member's target mass [kg]; a negative value clears it, so the
 * next start-up step captures it again (restarting from a new state). */
int aeros_dyn_set_mass_target(aeros_dyn_t h, double mass);
/* The mass-fixer scalars of one member, read and restored: the restart
 * attributes mass_target, lnr_last, lnr_cum of aeros_timestep_write_restart /
 * _read_restart (src/dynamics/aeros_timestep.f90:1303-1633).  A negative
 * mass_target clears the member's target (captured again at a start-up step). */
int aeros_dyn_member_counters(aeros_dyn_t h, int member, double *mass_target, double *lnr_last,
                              double *lnr_cum);
int aeros_dyn_set_member_counters(aeros_dyn_t h, int member, double mass_target, double lnr_last,
                                  double lnr_cum);

/* Zonal-mean statistics (src/aeros_diagnostics.f90:153-276): accumulate one
 * sample of the current state; read the running means of member `member`
 * as 7 arrays (nlat, nlev): u, v, temp, u'v', v'T', eke, T'^2, and 2 arrays
 * (nlat): ps, u_sfc.  `out` holds 7*nlat*nlev + 2*nlat doubles. */
int aeros_dyn_diag_accumulate(aeros_dyn_t h);
int aeros_dyn_diag_read(aeros_dyn_t h, int member, double *out, int *nsample);

/* Fastest linear gravity-wave speed [m/s] of the semi-implicit operator W
 * (src/dynamics/aeros_semiimp.f90:573-620). */
int aeros_dyn_gwspeed(aeros_dyn_t h, double *cmax);

/* Bind to a caller's CUDA stream; steps are replayed as CUDA graphs on it. */
int aeros_dyn_set_stream(aeros_dyn_t h, void *stream);

/* Number of this library's kernel launches issued since creation (a step
 * replayed from a graph counts each kernel node). */
int aeros_dyn_launch_count(aeros_dyn_t h, long long *count);

/* Launch-shape autotuner (no reference counterpart): times whole steps for
 * each candidate shape of the longitude FFTs (latitudes and threads per CTA),
 * the FP64 Legendre analysis (columns per CTA) and synthesis (latitudes per
 * CTA), the column kernel (threads per CTA, lanes per column), the
 * spectral kernel (warps per CTA; a warp per coefficient or, for 16 or 20
 * levels, a thread per real column) and, in the split form, the grid sizes of
 * the tensor-core kernels, keeps the fastest, restores the state and
 * re-captures the step graphs.  ms_before / ms_after: step time with the old and the chosen shapes.
 * With AEROS_TUNE_CACHE set to a file name, results are appended there and new
 * handles of the same GPU, grid, levels, ensemble size and precision start
 * from them.  Tune member handles before grouping them. */
int aeros_dyn_autotune(aeros_dyn_t h, int reps, double *ms_before, double *ms_after);
/* The shapes in use, in the order fs_lpb, fs_thr, fa_lpb, fa_thr, la_ct,
 * col_thr, spec_warps, col_lanes, ls_jt (0 = heuristic), spec_cols (0 a warp
 * per coefficient, 1 a thread per real column), sp_cps and sp_dft_cps (split
 * Legendre kernels and split DFT products: CTAs per SM over the grid, 2, 4, 8
 * or 16): the first n (0 <= n <= 12) are written to shape. */
int aeros_dyn_tune_get(aeros_dyn_t h, int *shape, int n);
/* Set the shapes (same order; n = 12, or 10 keeping the two split shapes),
 * each one the autotuner would try, and re-capture the step graphs.
 * AEROS_ERR_ARG for any other shape. */
int aeros_dyn_tune_set(aeros_dyn_t h, const int *shape, int n);

/* ======================================================================== */
/* Ensemble groups: several dyn handles (e.g. members of different          */
/* truncations and level counts) stepped by ONE CUDA graph launch per time  */
/* step.  The group records every handle's step launches and fuses them:   */
/* at each kernel of the step, the handles that run the same kernel share   */
/* one ragged launch (up to 4 handles per launch; each CTA finds its        */
/* handle, block index and grid in a descriptor table), so a step of 96     */
/* members in three truncations is about one launch per kernel type.  The   */
/* kernels the handles share get the launch shapes of the heaviest handle   */
/* (results do not depend on launch shapes).  A group with a physics hook,  */
/* or with AEROS_GROUP_FUSE=0 in the environment, makes each handle's own   */
/* step graph a branch of the group's graph instead.  Handles must be fully */
/* configured (state, forcing, phis) and at the same step count; while in a */
/* group, step them only through the group.  No reference counterpart: the */
/* reference steps one configuration per process.                          */
/* ======================================================================== */
int aeros_group_create(aeros_group_t *g, aeros_dyn_t *handles, int n);
int aeros_group_destroy(aeros_group_t g);
int aeros_group_set_stream(aeros_group_t g, void *stream);
int aeros_group_step(aeros_group_t g, int nsteps);
int aeros_group_step_async(aeros_group_t g, int nsteps);
int aeros_group_sync(aeros_group_t g);
int aeros_group_launch_count(aeros_group_t g, long long *count);
/* fused: 1 when the launches are fused, 0 for one branch per handle;
 * kernels_startup / kernels_step: kernel launches of the start-up and of a
 * regular step (any pointer may be NULL). */
int aeros_group_info(aeros_group_t g, int *fused, long long *kernels_startup, long long *kernels_step);

/* ======================================================================== */
/* Differentiation: adjoints of the transforms and of the step              */
/* (no reference counterpart: aeros has no adjoint).  Inner products are     */
/* the Euclidean ones of the arrays: sum of grid values, and sum over        */
/* (l, m) of Re(conj(a) b) for spectral arrays; m = 0 imaginary parts are    */
/* not degrees of freedom.  Same argument conventions (host or device        */
/* pointers, batches) as the forward transforms.                             */
/* ======================================================================== */
/* coeffs_ad = synthesis^T field_ad */
int aeros_sht_synthesis_ad(aeros_sht_t h, const double *field_ad, double *coeffs_ad, int nbatch);
/* field_ad = analysis^T coeffs_ad */
int aeros_sht_analysis_ad(aeros_sht_t h, const double *coeffs_ad, double *field_ad, int nbatch);
/* (slm_ad, tlm_ad) = synthesis_vec^T (vth_ad, vph_ad) */
int aeros_sht_synthesis_vec_ad(aeros_sht_t h, const double *vth_ad, const double *vph_ad, double *slm_ad,
                               double *tlm_ad, int nbatch);
/* (vth_ad, vph_ad) = analysis_vec^T (slm_ad, tlm_ad) */
int aeros_sht_analysis_vec_ad(aeros_sht_t h, const double *slm_ad, const double *tlm_ad, double *vth_ad,
                              double *vph_ad, int nbatch);

/* Complex entries of a packed state: M (3 nlev + 1) nlm, laid out as
 * vor (M, nlev, nlm) | div | temp | lnps (M, nlm) -- the order of
 * aeros_dyn_set_state's four arrays, concatenated. */
int aeros_dyn_state_size(aeros_dyn_t h, long long *n);

/* Adjoint of the next step (the one aeros_dyn_step(h, 1) would take from the
 * current state; the state is left unchanged).  In: adjoints of the post-step
 * old slot (the RAW-filtered X^n) and now slot (X^(n+1)), packed.  Out:
 * adjoints of the pre-step old (X^(n-1)) and now (X^n) slots, packed, and per
 * member d/dk_a, d/ddT_y (any output may be NULL). */
int aeros_dyn_step_ad(aeros_dyn_t h, const double *old_ad_in, const double *now_ad_in, double *old_ad_out,
                      double *now_ad_out, double *ka_ad, double *dty_ad);

/* Forward half of the window pair: step nsteps from the current state,
 * keeping a checkpoint every ckpt_every steps, and return per member
 * J = (1/nsteps) sum_{n=1..nsteps} sum_k int (u^2 + v^2)/2 dp_k/g dA [J],
 * the window mean of the kinetic part of aeros_budget's energy. */
int aeros_dyn_window_forward(aeros_dyn_t h, int nsteps, int ckpt_every, double *J);

/* Backward half: gradient of sum_e J_e with respect to the state at the start
 * of the window (packed, now and old slots; the old slot's is zero when the
 * window starts at step 0) and to each member's k_a and dT_y.  Segments are
 * recomputed from the checkpoints; the handle is left at the end of the window. */
int aeros_dyn_window_backward(aeros_dyn_t h, double *now_ad, double *old_ad, double *ka_ad, double *dty_ad);

/* Message of the last failed call on the calling thread (thread-local storage,
 * valid until that thread's next failing call). */
const char *aeros_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* AEROS_GPU_H */
