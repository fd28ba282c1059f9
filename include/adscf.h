/*
 * adscf.h -- C ABI of the GB300 (sm_103a) SCF inner-loop library.
 *
 * The library replaces the compute core of ADSCF's Fortran 90 module
 * procedures.  Every entry point below names the reference routine it
 * stands in for (file:line within the ADSCF tree).  The Fortran drivers
 * keep their input decks, SCF loop and output; they bind these functions
 * through iso_c_binding.
 *
 * Conventions
 *  - Plain C: opaque handles, plain pointers and sizes, int status returns.
 *    Nothing here prints, exits or throws.
 *  - Field arrays are [species][z][y][x] FP64, the same linear order as the
 *    reference's Fortran (x,y,z,species).  Films and brushes include both
 *    wall planes, z = 0..gz.
 *  - Host pointers are caller-owned; functions without the _dev suffix copy
 *    host data in and out.  *_dev variants take device pointers.
 *  - A context owns its device buffers and its CUDA stream.  One context per
 *    host thread; a context is not safe for concurrent use.
 */
#ifndef ADSCF_H
#define ADSCF_H

#ifdef __cplusplus
extern "C" {
#endif

#define ADSCF_ABI_VERSION 2
#define ADSCF_MAX_BLOCKS 16   /* blocks of a linear multiblock chain */

#if defined(__GNUC__)
#define ADSCF_API __attribute__((visibility("default")))
#else
#define ADSCF_API
#endif

/* status codes (the reference has none: it prints and stops) */
enum {
  ADSCF_OK = 0,
  ADSCF_E_ARG = 1,        /* invalid argument / unsupported shape          */
  ADSCF_E_CUDA = 2,       /* CUDA runtime error                            */
  ADSCF_E_PIVOT = 3,      /* zero tridiagonal pivot ("TriDiag Error",
                             Film_3D/.../mod_realspace.f90:194-207)         */
  ADSCF_E_NONFINITE = 4,  /* non-finite Q, density or field                */
  ADSCF_E_TIMEOUT = 5,    /* bounded device wait expired                   */
  ADSCF_E_OOM = 6,        /* device allocation failed                      */
  ADSCF_E_STATE = 7,      /* call not valid for this context / state       */
  ADSCF_E_TOO_LARGE = 8   /* problem exceeds the fixed scratch of the
                             allocation-free entry point                  */
};

enum { ADSCF_BULK = 0, ADSCF_FILM_1D = 1, ADSCF_FILM_3D = 2, ADSCF_BRUSH = 3 };
/* precision policy: FP64 everywhere, or FP32 propagators/FFTs/line sweeps
 * with FP64 Q, free energy, compensated density accumulation and mixing   */
enum { ADSCF_FP64 = 0, ADSCF_SPLIT = 1 };
/* mixing_type as in main_diblock.f90:44 */
enum { ADSCF_MIX_SIMPLE = 1, ADSCF_MIX_LAMBDA = 2, ADSCF_MIX_ANDERSON = 3 };

typedef struct adscf_params {
  int geometry;             /* ADSCF_BULK, ADSCF_FILM_1D, ADSCF_FILM_3D, ADSCF_BRUSH */
  int gx, gy, gz;           /* bulk: grid points; films/brush: gz >= 2 intervals, planes 0..gz */
  double sizex, sizey, sizez;
  double ds;                /* uniform contour step (input_general)          */
  const double *dss;        /* optional [ns+1] contour steps, dss[0] = 0
                               (Brush mod_homopolymer.f90:98-115); NULL = ds */
  int ns;                   /* contour steps when dss != NULL                */
  int n_a;                  /* contour node of the A-B junction (dss != NULL) */
  double block_length[2];   /* f_A, f_B; segments = nint(f/ds)
                               (mod_diblock.f90:74)                           */
  int ensemble;             /* 1 canonical, 2 grand canonical                */
  double rho, mu;           /* C and mu_scf of input_general                 */
  double kappa, chi;        /* input_interactions                            */
  double monomer_volume[2];
  int precision;            /* ADSCF_FP64 or ADSCF_SPLIT                      */
  int mixing_type;          /* ADSCF_MIX_*                                    */
  int mixing_dim;           /* Anderson history m (reference: 2)             */
  double lambda;            /* lambda / lam_mix / lammax                     */
  double lam_warm;          /* Anderson warm-up step (reference lam00 1e-3)  */
  int warm_iters;           /* Anderson for iter > warm_iters (>= mixing_dim) */
  const double *dz;         /* films/brush: [gz+1] mesh steps, dz[0] = 0     */
  int int_scheme;           /* films/brush: 0 rectangle, 1 trapezoid         */
  int int_span;             /* 0: Film_3D integrator (full), 1: Film_1D/Brush
                               integrator (interior intervals only)          */
  const double *ext_potential; /* films/brush: [types][gz+1] wall potential
                               added inside Calculate_Mean_Ext_Fields; NULL=0 */
  double ww;                /* brush: w = ww*phi + U (mod_virial_expansion) */
  const double *graft;      /* brush: [gz+1] grafting distribution q-dag_0   */
  /* bulk linear block sequence (Initialize_Multiblock / Propagate_Multiblock,
     Polymer_Modules/mod_multiblock.f90:46-180; Propagate_Triblock and the
     homopolymer are its 3- and 1-block cases): nblocks > 0 replaces the
     diblock of block_length.  Block k has nint(blocks[k]/ds) segments of
     monomer type block_types[k] (0 = A, 1 = B); densities are per type, the
     sum of the block distributions of that type.  At most ADSCF_MAX_BLOCKS. */
  int nblocks;
  const double *blocks;
  const int *block_types;
} adscf_params;

typedef struct adscf_ctx adscf_ctx;

/* chain quantities of Propagate_Diblock / Propagate_Homopolymer */
typedef struct adscf_chain_result {
  double Qsum;     /* single-chain partition function (dvol * sum q_N)   */
  double logQ;
  double mu;       /* chemical potential                                  */
  double rho;      /* polymer concentration                               */
  double energy;   /* chain energy term of the ensemble                   */
} adscf_chain_result;

/* one Calculate_Saddle_Point loop body (main_diblock.f90:410-429) */
typedef struct adscf_iter_result {
  double accuracy;      /* Check_Accuracy: sum (phi_old - phi_new)^2       */
  double free_energy;   /* [chain - dvol sum(phi w) + interaction] / (rho V) */
  double Qsum, logQ, mu, rho;
  double lambda;        /* mixing step used                                */
  int iter;             /* 1-based iteration index                         */
  int status;
} adscf_iter_result;

/* ---- context ----------------------------------------------------------
 * Initialize (Bulk_3D_FFT/General_Routines/sub_wrap.f90:8-40):
 * Initialize_Fourier + Calculate_Laplace + Calculate_Volume_Parameters
 * (mod_fourier.f90:49-54,152-198), Initialize_Diblock (mod_diblock.f90:46-88),
 * Initialize_Interactions (mod_FloryHuggins.f90:37-66); films: generate_mesh
 * (Film_3D/.../mod_realspace.f90:222-265) is done by the caller, who passes
 * dz.  Finish (sub_wrap.f90:48-58) is adscf_ctx_destroy.                   */
ADSCF_API int adscf_ctx_create(const adscf_params *params, adscf_ctx **ctx);
ADSCF_API int adscf_ctx_destroy(adscf_ctx *ctx);
ADSCF_API const char *adscf_status_string(int status);
ADSCF_API const char *adscf_last_error(const adscf_ctx *ctx);
ADSCF_API int adscf_abi_version(void);
/* number of points of one species field ([z][y][x], walls included) */
ADSCF_API long long adscf_field_points(const adscf_ctx *ctx);
/* contour steps (segments) and A-block steps of the chain */
ADSCF_API int adscf_contour_info(const adscf_ctx *ctx, int *ns, int *n_a);

/* ---- propagator -------------------------------------------------------
 * Calculate_Expfield (Bulk_3D_FFT/General_Routines/mod_propagate.f90:22-32)
 * + Propagate_Diblock (Bulk_3D_FFT/Polymer_Modules/mod_diblock.f90:100-173;
 * films Film_CK_AD/Film_1D/Polymer_Modules/mod_diblock.f90:110-195,
 * Film_3D :105-182).  field [2][npts] in, density [2][npts] out (by
 * monomer type, main_diblock.f90:277-283).                                 */
ADSCF_API int adscf_propagate_diblock(adscf_ctx *ctx, const double *field,
                            double *density, adscf_chain_result *out);
ADSCF_API int adscf_propagate_diblock_dev(adscf_ctx *ctx, const double *d_field,
                                double *d_density, adscf_chain_result *out);

/* Propagate_Homopolymer (Brush_CK_AD/Polymer_Modules/mod_homopolymer.f90:
 * 181-259): single-species field [npts], density [npts].                   */
ADSCF_API int adscf_propagate_homopolymer(adscf_ctx *ctx, const double *field,
                                double *density, adscf_chain_result *out);

/* Propagate_Step: one contour step on one propagator in place.
 *  bulk : prop <- E IFFT(exp(-k^2 ds) FFT(E prop)), E = expfield
 *         (mod_propagate.f90:40-68; expfield from Calculate_Expfield);
 *  films: Crank-Nicolson / Douglas ADI step with the given field and ds
 *         (Film_1D/.../mod_realspace.f90:24-79, Film_3D :22-140,
 *         Brush_CK_AD/Geometry_Modules/mod_realspace.f90:26-79);
 *         `aux` is the field w, `ds` the step (<= 0: params ds).          */
ADSCF_API int adscf_propagate_step(adscf_ctx *ctx, double *prop, const double *aux,
                         double ds);

/* Real2Fourier (scaled 1/N) and Fourier2Real (unnormalised), bulk only,
 * mod_fourier.f90:75-105.  Spectrum is the r2c half spectrum
 * [gz][gy][gx/2+1] of interleaved (re, im) doubles.                         */
ADSCF_API int adscf_real2fourier(adscf_ctx *ctx, const double *prop, double *spectrum);
ADSCF_API int adscf_fourier2real(adscf_ctx *ctx, const double *spectrum, double *prop);

/* integrator (Film_3D/.../mod_realspace.f90:267-281, Brush
 * mod_adaptive.f90:124-143); bulk: dvol * sum.                              */
ADSCF_API int adscf_integrator(adscf_ctx *ctx, const double *integrand, double *integral);

/* ---- interactions -----------------------------------------------------
 * Calculate_Mean_Fields (mod_FloryHuggins.f90:104-129) / films
 * Calculate_Mean_Ext_Fields (Film_1D/.../mod_FloryHuggins.f90:140-167) with
 * params.ext_potential as the wall potential; brush w = ww phi + U
 * (mod_virial_expansion.f90:111-137).                                       */
ADSCF_API int adscf_mean_fields(adscf_ctx *ctx, const double *density, double *field);
/* Interaction_Energy (mod_FloryHuggins.f90:74-96) */
ADSCF_API int adscf_interaction_energy(adscf_ctx *ctx, const double *density,
                             double *energy);

/* ---- monomeric solvent --------------------------------------------------
 * Update_Solvent (Bulk_3D_FFT/Polymer_Modules/mod_solvent.f90:85-110) on a
 * bulk context's grid: distribution = exp(-field), Qsum = dvol sum, then
 * canonical (ensemble 1): density = rho V distribution / Qsum,
 *   mu = log(rho V / Qsum), energy = rho V (mu - 1);
 * grand canonical (2): density = exp(mu) distribution,
 *   rho = dvol sum(density) / V, energy = -rho V.
 * field, density and distribution (optional, NULL to skip) are [npts];
 * rho and mu are read or written as the ensemble requires.                 */
ADSCF_API int adscf_update_solvent(adscf_ctx *ctx, const double *field, int ensemble, double *rho,
                                   double *mu, double *Qsum, double *energy, double *density,
                                   double *distribution);

/* ---- mixing -----------------------------------------------------------
 * Mix_Fields (main_diblock.f90:315-372) with Mixing_Simple / Mixing_Lambda /
 * Mixing_Anderson (mod_iterate.f90:27-150), history kept on the device
 * across calls.  field: in x_k, out x_{k+1}; dfield: r_k.                   */
ADSCF_API int adscf_mix(adscf_ctx *ctx, double *field, const double *dfield, int iter);
ADSCF_API int adscf_mix_dev(adscf_ctx *ctx, double *d_field, const double *d_dfield,
                  int iter);
/* forget the mixing history (next call behaves as iter == 1) */
ADSCF_API int adscf_mix_reset(adscf_ctx *ctx);

/* ---- whole SCF iteration on the device --------------------------------
 * Loop body of Calculate_Saddle_Point (main_diblock.f90:410-429): densities,
 * Check_Accuracy, mean fields, Mix_Fields, all device resident.  The whole
 * iteration is replayed from a CUDA graph.  adscf_set_field loads x_1 and
 * resets the iteration counter and density history.                       */
ADSCF_API int adscf_set_field(adscf_ctx *ctx, const double *field);
ADSCF_API int adscf_set_density(adscf_ctx *ctx, const double *density);
ADSCF_API int adscf_get_field(adscf_ctx *ctx, double *field);     /* current x_k   */
ADSCF_API int adscf_get_density(adscf_ctx *ctx, double *density); /* newest phi    */
/* n iterations; result describes the last one.  Stops early when
 * accuracy <= tol (tol < 0: never).                                        */
ADSCF_API int adscf_scf_run(adscf_ctx *ctx, int n_iter, double tol,
                  adscf_iter_result *out);
/* one iteration with host buffers: field in (x_k) -> field out (x_{k+1}),
 * density out (phi[x_k]); the call a Fortran SCF loop makes per iteration.
 * Page-locked buffers (cudaHostAlloc / cudaHostRegister) are copied by DMA
 * directly; pageable ones go through the context's pinned staging buffer. */
ADSCF_API int adscf_scf_iteration(adscf_ctx *ctx, double *field, double *density,
                        adscf_iter_result *out);

/* ---- streams and asynchronous stages ---------------------------------
 * Run all further work of the context on the caller's CUDA stream
 * (cudaStream_t passed as void*; NULL restores the context's own stream).
 * No reference counterpart: the reference is synchronous CPU code.        */
ADSCF_API int adscf_set_stream(adscf_ctx *ctx, void *cuda_stream);
/* Enqueue `repeats` runs of one stage on the context stream without any
 * host synchronisation, starting from the device-resident field:
 *   ADSCF_STAGE_ITERATION  whole SCF iteration (graph replay)
 *   ADSCF_STAGE_PROPAGATE  both chains, all contour steps (no contour sum)
 *   ADSCF_STAGE_CONTOUR    contour integral of the densities and Q
 *   ADSCF_STAGE_UPDATE     closure, mean fields, residual, mixing solve+mix */
enum { ADSCF_STAGE_ITERATION = 0, ADSCF_STAGE_PROPAGATE = 1,
       ADSCF_STAGE_CONTOUR = 2, ADSCF_STAGE_UPDATE = 3 };
ADSCF_API int adscf_enqueue(adscf_ctx *ctx, int stage, int repeats);
/* kernel launches one run of a stage makes (for launch accounting) */
ADSCF_API int adscf_stage_launches(const adscf_ctx *ctx, int stage);
/* Bound of one pipeline wait of the TMA-fed bulk passes, in polls of its
 * mbarrier (default 2^22, restored by polls < 0; 0 makes every wait give up
 * at once).  A wait that runs out sets a device flag; the kernel drains its
 * copies in flight and returns, and the next result-reading call returns
 * ADSCF_E_TIMEOUT.  No reference counterpart (failure detection of the
 * device pipeline; the reference's only failure stops are the tridiagonal
 * pivot and the non-finite accuracy checks).                              */
ADSCF_API int adscf_set_wait_limit(adscf_ctx *ctx, int polls);

/* ---- pass-kernel autotuner (bulk) ----------------------------------------
 * No reference counterpart.  At context creation every available kernel for
 * each line pass of the double step -- Y and Z: plain, persistent or
 * TMA-fed; X: plain, persistent, or the fused plane pass that also does Yi
 * and Yf (then the Y choice is moot) -- is timed on the context's own buffers
 * and the fastest plan kept (cached per device, grid and precision; the
 * environment variable ADSCF_AUTOTUNE=0 keeps the default plan instead:
 * the TMA-fed Y and Z passes with the fused plane pass where they exist,
 * else the persistent, else the plain kernels).
 * All plans compute the same arithmetic: results do not depend on the choice.
 * adscf_tuning writes the plan and the per-candidate timings as text;
 * adscf_set_pass_plan pins a plan (ADSCF_E_ARG if unavailable).           */
enum { ADSCF_PASS_PLAIN = 0, ADSCF_PASS_PERSISTENT = 1, ADSCF_PASS_TMA = 2,
       ADSCF_PASS_FUSED = 3 /* x only: one plane pass for Yi + X + Yf */ };
ADSCF_API int adscf_tuning(const adscf_ctx *ctx, char *buf, int len);
ADSCF_API int adscf_set_pass_plan(adscf_ctx *ctx, int y, int z, int x);

/* ---- ADI sweep autotuner (Film_3D, FP32 sweeps) -------------------------
 * No reference counterpart.  Each Douglas ADI sweep (x, y, z lines) runs on
 * a warp solver with G lanes per line and K points per lane -- for the y and
 * z lines optionally staged through shared memory in tiles of 32 lines, so
 * that global accesses are coalesced -- or on one thread per line.  At
 * context creation every shape that fits the lines is timed on the
 * context's buffers and each sweep keeps its fastest (cached per device and
 * grid; ADSCF_AUTOTUNE=0 keeps the defaults).  Shapes order the FP32
 * line-solve arithmetic differently, so results agree to FP32 rounding, not
 * bit for bit.  On a square plane whose x and y sweeps chose one unstaged
 * shape (16 or 8 lanes, 2 or 4 points each), the two sweeps as one kernel
 * per plane and chain (the plane held in shared memory, the same arithmetic)
 * are timed too and kept if faster ("xy=fused").  adscf_tuning reports the
 * choice and the timings ("GxK", "s" for staged); adscf_set_adi_plan pins
 * lanes per line for each sweep (0: one thread per line), staging (mask: 2 y,
 * 4 z) and the fused x + y kernel (mask 8); ADSCF_E_ARG if no shape matches,
 * ADSCF_E_STATE for other contexts.                                        */
ADSCF_API int adscf_set_adi_plan(adscf_ctx *ctx, int x_lanes, int y_lanes, int z_lanes, int staged);

/* ---- differentiation (bulk, FP64 context, canonical ensemble) ----------
 * No counterpart in the reference, which has no derivatives; it replaces
 * the reference's practice of differencing converged free energies of
 * neighbouring box sizes (main_diblock.f90's Calculate_Energy, re-run).
 * adscf_forward: free energy per chain at the host fields [2][gz][gy][gx]
 * without mixing -- chain term log(rho V/Q) - 1 minus dvol sum(phi w) plus
 * Interaction_Energy (mod_FloryHuggins.f90:74-96), over rho V, with phi
 * from Propagate_Diblock (mod_diblock.f90:100-173) -- keeping every
 * propagator slice on the device.
 * adscf_backward: reverse-mode adjoint of that discrete free energy at the
 * same fields: grad[0..2] = dF/dL_x, dF/dL_y, dF/dL_z (cell stress),
 * grad[3] = dF/dchi.  Exact for the discretisation (pseudo-spectral steps,
 * trapezoid contour), so at a converged saddle point grad[0..2] are the
 * derivatives of the equilibrium free energy.  Any other propagating call
 * on the context between the two returns ADSCF_E_STATE.                  */
ADSCF_API int adscf_forward(adscf_ctx *ctx, const double *field, double *free_energy);
ADSCF_API int adscf_forward_dev(adscf_ctx *ctx, const double *d_field, double *free_energy);
ADSCF_API int adscf_backward(adscf_ctx *ctx, double *grad);
/* Checkpointing of the FP64 bulk forward/backward pair (no counterpart in
 * the reference, which stores every node): every = K > 0 keeps the states
 * of both chains at nodes kK and at the mirror nodes Ns - (k+1)K + 1 and
 * recomputes segments of K steps when the contour integral and the reverse
 * sweep need them; every < 0 picks K = ceil(sqrt(Ns)).  The context then
 * releases its Ns + 1 propagator slices (storage 2 ceil(Ns/K) + 2K + 4
 * slices) and its SCF / propagation calls return ADSCF_E_STATE until
 * every = 0 restores them.  A forward made before the call cannot be
 * paired with a later backward.  Results equal the stored-slice pass up to
 * the summation order of the contour integral.                            */
ADSCF_API int adscf_set_adjoint_checkpoint(adscf_ctx *ctx, int every);
/* ---- dynamic density functional theory (bulk, two monomer types) -----
 * The DDFT step of the multiblock driver (Bulk_3D_FFT/Main_Multiblock/
 * main_multiblock.f90).
 * adscf_ddft_set_mobility: Read_Mobilities (:441-506) from the rows of
 *   input_mobilities: table[nq][3] = (Lambda_AA, Lambda_AB, Lambda_BB) at
 *   q = (i+1) dq; mobility_qq(k) = min(|k|^2 Lambda(|k|), wcutoff) with the
 *   reference's interpolation between rows.
 * adscf_ddft_rhs: d rho / dt = -IFFT(mobility_qq FFT(mu)) for a host
 *   mu[2][npts] (:836-861), into ddensity[2][npts].
 * adscf_conjugate_fields: Get_Conjugate_Fields (:566-640) -- the context's
 *   mixing iterates its current field until max |phi[w] - density| <=
 *   accuracy / 2 (warm-up restarted on every call, as the reference's
 *   iter_status); *status = 0 converged, 1 within accuracy but not half of
 *   it, 2 not found (ADSCF_E_NONFINITE when the accuracy is >= 0.1 or not
 *   finite, where the reference stops).  adscf_get_field then returns the
 *   conjugate field.  The reference uses Anderson mixing with lambda 0.5,
 *   accuracy 1e-3 and 2000 iterations.
 * adscf_ddft_step: DDFT_Timestep_Euler (:794-880) on density[2][npts]
 *   (in/out): conjugate fields, mu = mean fields of the density minus the
 *   conjugate field, the Euler step with timestep, the floor at 1e-4 when
 *   floor_density, and the conjugate fields of the new density (*status as
 *   above; with floor_density and status >= 1 the density becomes that of
 *   the field found).  No counterpart of these four entry points is a
 *   separate reference procedure except as cited.                         */
ADSCF_API int adscf_ddft_set_mobility(adscf_ctx *ctx, int nq, double dq, const double *table, double wcutoff);
ADSCF_API int adscf_ddft_rhs(adscf_ctx *ctx, const double *mu, double *ddensity);
ADSCF_API int adscf_conjugate_fields(adscf_ctx *ctx, const double *density, double accuracy, int itermax,
                                     int *status, int *iterations);
ADSCF_API int adscf_ddft_step(adscf_ctx *ctx, double *density, double timestep, int floor_density,
                              double accuracy, int itermax, int *status);
/* Films and brushes (any precision): adscf_forward gives the free energy
 * per chain at the host fields (the film Calculate_Energy with the external
 * term); adscf_backward_surface then gives dF/dchi (brush: dF/dww) and the
 * gradient with respect to the wall potential, dF_dU[c][z] for every type c
 * and plane z = 0..gz (the ext_potential array of adscf_params).  At fixed
 * fields the densities do not depend on U, so the gradient is the
 * plane-weighted density over rho V.                                      */
ADSCF_API int adscf_backward_surface(adscf_ctx *ctx, double *dF_dchi, double *dF_dU);

/* New box side lengths for a bulk context (unit-cell relaxation): the
 * k-space factors of Calculate_Laplace (mod_fourier.f90:165-198) and the
 * volume terms are recomputed in place; fields, densities and the mixing
 * history are kept.  No reference counterpart: the reference fixes the box
 * at start-up.                                                            */
ADSCF_API int adscf_set_box(adscf_ctx *ctx, double sizex, double sizey, double sizez);

/* FP64 free energy per chain at the context's current device-resident SCF
 * field (bulk, canonical).  A split context iterates in FP32/FP64-split
 * precision; at a converged field F is stationary in the densities, so one
 * FP64 evaluation there (on an FP64 sibling context, created on first use)
 * gives the saddle free energy to second order in the remaining field
 * error.  Fills free_energy, Qsum, logQ, mu, rho and iter of `out`.  No
 * reference counterpart (the reference is FP64 throughout).               */
ADSCF_API int adscf_free_energy_fp64(adscf_ctx *ctx, adscf_iter_result *out);

/* ---- batches of independent bulk instances ------------------------------
 * No single reference counterpart: the reference runs a phase-diagram or
 * box-size scan as separate invocations of the bulk driver
 * (Bulk_3D_FFT/Main_Diblock_Melt/main_diblock.f90), one parameter set each.
 * A batch holds n bulk instances (geometry ADSCF_BULK, one precision, any
 * grid of 2/3/5 factors, box, ds, block lengths, chi, kappa, mixing) and
 * advances all of them by one SCF iteration per step: one launch per line
 * pass and contour step over every instance still on its contour, batched
 * closure, Anderson solve and mixing with per-instance histories, captured as
 * one CUDA graph.  Fields and densities are packed: instance i occupies
 * [2][gz_i][gy_i][gx_i] doubles starting at adscf_batch_offset(b, i);
 * adscf_batch_offset(b, n) is the total.  adscf_batch_scf_run stops early
 * once every instance's accuracy is <= tol (tol < 0: run n_iter) and fills
 * out[n].                                                                 */
typedef struct adscf_batch adscf_batch;
ADSCF_API int adscf_batch_create(const adscf_params *params, int n, adscf_batch **out);
ADSCF_API int adscf_batch_destroy(adscf_batch *b);
ADSCF_API const char *adscf_batch_last_error(const adscf_batch *b);
ADSCF_API long long adscf_batch_offset(const adscf_batch *b, int i);
ADSCF_API int adscf_batch_set_fields(adscf_batch *b, const double *fields);
ADSCF_API int adscf_batch_get_fields(adscf_batch *b, double *fields);
ADSCF_API int adscf_batch_get_densities(adscf_batch *b, double *densities);
ADSCF_API int adscf_batch_scf_run(adscf_batch *b, int n_iter, double tol, adscf_iter_result *out);
ADSCF_API int adscf_batch_set_stream(adscf_batch *b, void *cuda_stream);
/* enqueue `repeats` batch iterations without host synchronisation */
ADSCF_API int adscf_batch_enqueue(adscf_batch *b, int repeats);
ADSCF_API int adscf_batch_results(adscf_batch *b, adscf_iter_result *out);
/* kernel launches of one batch iteration */
ADSCF_API int adscf_batch_launches(const adscf_batch *b);
/* FP64 bulk batches (canonical): free energy per chain of every instance at
 * the packed host fields (as adscf_forward), then the reverse-mode adjoint
 * of every instance in one sweep: grad[4 i + 0..3] = dF/dL_x, dF/dL_y,
 * dF/dL_z, dF/dchi of instance i (as adscf_backward).                      */
ADSCF_API int adscf_batch_forward(adscf_batch *b, const double *fields, double *free_energy);
ADSCF_API int adscf_batch_backward(adscf_batch *b, double *grad);

/* Measurement helper of the benchmark, no reference counterpart: copy
 * bandwidth (read + write bytes per second, in GB/s) of two buffers of
 * `bytes` each (1 MiB .. 256 MiB) on the current device: one launch
 * copies the buffer `reps` times after a launch that copies it twice;
 * below half the L2 size both buffers stay L2-resident, so this is the L2
 * bandwidth a streaming kernel sees.                                       */
ADSCF_API int adscf_probe_l2_copy(long long bytes, int reps, double *gbs);

/* ---- allocation-free propagator step ----------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory (a pre-partitioned or quota-limited GPU, a driver that owns every
 * device buffer, code paths where cudaMalloc's implicit synchronisation is
 * not allowed): one FP64 bulk propagator step, prop <- E IFFT(exp(-k^2 ds)
 * FFT(E prop)) with E = expfield, on caller-owned device buffers d_prop
 * [gz][gy][gx] (in/out) and d_expfield, enqueued on `stream` (cudaStream_t
 * as void*).  It calls no allocator: plan, tables and spectrum live in one
 * file-scope static device array of about 6.6 MB, reserved on a device when
 * the library's device code loads there (under CUDA's default lazy loading,
 * at the first call on that device; ADSCF_E_OOM if that fails) and held
 * until exit.  Limits: gx*gy*gz <= 262144, each axis <= 512 and a product of
 * 2, 3 and 5, gx*gy <= 65536; larger problems return ADSCF_E_TOO_LARGE.  The
 * first call on a device sets the array up (cudaGetSymbolAddress, kernel
 * attributes), and a call with a new grid, box or ds rebuilds the tables in
 * the array with a stream synchronisation; both return ADSCF_E_STATE while
 * the stream is capturing, so make them before any stream capture.  All
 * calls share the array: calls whose kernels overlap on the GPU race, and a
 * rebuild replaces the tables that earlier enqueued or recorded work reads.
 * Order the calls on one stream.                                           */
ADSCF_API int adscf_propagate_step_noalloc(int gx, int gy, int gz, double sizex,
                                           double sizey, double sizez, double ds,
                                           double *d_prop, const double *d_expfield,
                                           void *stream);

#ifdef __cplusplus
}
#endif
#endif /* ADSCF_H */
