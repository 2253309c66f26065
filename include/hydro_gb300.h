/*
 * hydro_gb300.h -- C ABI of libhydro_gb300.so, the GB300 (sm_103a) drop-in for
 * HydroCODE's Eulerian Godunov/GRP scheme call (1D and 2D structured,
 * single-fluid, ideal gas).
 *
 * Part 1 is the drop-in boundary: the four scheme entry points with the
 * signatures, argument meaning, ownership and side effects of the reference's
 * src/include/finite_volume.h.  Inputs come from the global `double config[]`
 * (defined by the caller, as the reference's drivers do; the library carries a
 * weak fallback definition), the caller owns every array, and results are
 * written back exactly where the reference writes them.
 *
 * Part 2 is a native API with no reference counterpart: a device-resident 2D
 * solver handle (used by the tests and the benchmark), the precision/guess
 * form selector and error reporting.
 *
 * All calls are synchronous, run on the current CUDA device and, like the
 * reference, are not re-entrant (one global config[]).
 */
#ifndef HYDRO_GB300_H
#define HYDRO_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#ifndef N_CONF
#define N_CONF 400
#endif

/* The caller's configuration array (reference: src/include/var_struc.h:44,
 * defined in src/hydrocode_2D/hydrocode.c:123 and src/hydrocode_1D/hydrocode.c:111).
 * Indices follow the reference's doc/config.csv; this library additionally reads
 *   config[300]  precision/guess form of the 2D scheme (HYDRO_FORM_*; INFINITY or
 *                absent = HYDRO_FORM_FP64, the reference's arithmetic);
 *   config[301]  interface GRP solver of the 2D schemes (HYDRO_SOLVER_*; INFINITY or
 *                absent = HYDRO_SOLVER_Q1D, the one the reference calls). */
extern double config[];

/* Same member order as the reference's struct cell_var_stru
 * (src/include/var_struc.h:61-74, single-fluid build). */
struct cell_var_stru {
    double **E;
    double **RHO, **U, **V, **P;
    double *d_rho, *d_u, *d_v, *d_p;
    double **s_rho, **s_u, **s_v, **s_p;
    double **t_rho, **t_u, **t_v, **t_p;
    double **rhoIx, **uIx, **vIx, **pIx;
    double **rhoIy, **uIy, **vIy, **pIy;
    double **F_rho, **F_e, **F_u, **F_v;
    double **G_rho, **G_e, **G_u, **G_v;
};

/* ---- Part 1: drop-in scheme entry points --------------------------------- */

/* 1D first-order Godunov scheme with the exact Riemann solver.
 * Replaces src/finite_volume/godunov_solver_EUL_source.c:27 (declared at
 * src/include/finite_volume.h:33).  CV.RHO/U/P/E[k][j], k < *N_plot. */
void Godunov_solver_EUL_source(const int m, struct cell_var_stru CV, double *cpu_time, int *N_plot,
                               double time_plot[]);

/* 1D second-order direct Eulerian GRP scheme.
 * Replaces src/finite_volume/grp_solver_EUL_source.c:27 (finite_volume.h:37). */
void GRP_solver_EUL_source(const int m, struct cell_var_stru CV, double *cpu_time, int *N_plot,
                           double time_plot[]);

/* 1D first-order Lagrangian Godunov scheme: cells keep their masses, the
 * nodes X[k][0..m] move with the star velocity (X[0] holds the initial nodes).
 * Replaces src/finite_volume/godunov_solver_LAG_source.c:28 (finite_volume.h:16). */
void Godunov_solver_LAG_source(const int m, struct cell_var_stru CV, double *X[], double *cpu_time, int *N_plot,
                               double time_plot[]);

/* 1D second-order Lagrangian GRP scheme.
 * Replaces src/finite_volume/grp_solver_LAG_source.c:28 (finite_volume.h:20). */
void GRP_solver_LAG_source(const int m, struct cell_var_stru CV, double *X[], double *cpu_time, int *N_plot,
                           double time_plot[]);

/* 2D unsplit GRP scheme.  CV[k].RHO/U/V/P/E[j][i] (x-major), k < N_T.
 * Replaces src/finite_volume/grp_solver_2D_EUL_source.c:75 (finite_volume.h:43-44). */
void GRP_solver_2D_EUL_source(const int m, const int n, struct cell_var_stru *CV, double **X, double **Y,
                              double *cpu_time, const char *problem, int N_T, int *N_plot, double time_plot[]);

/* 2D dimension-split GRP scheme.
 * Replaces src/finite_volume/grp_solver_2D_split_EUL_source.c:75 (finite_volume.h:48-49). */
void GRP_solver_2D_split_EUL_source(const int m, const int n, struct cell_var_stru *CV, double **X, double **Y,
                                    double *cpu_time, const char *problem, int N_T, int *N_plot,
                                    double time_plot[]);

/* ---- Part 2: native API (no reference counterpart) ------------------------ */

enum {
    HYDRO_FORM_FP64 = 0,         /* reference arithmetic in FP64 (parity form) */
    HYDRO_FORM_FP32 = 1,         /* FP32 state and fluxes, FP64 near-vacuum Newton */
    HYDRO_FORM_FP32_LEARNED = 2  /* FP32 form with the learned Newton starting pressure */
};

/* Interface GRP solver of GRP_2D_flux (src/flux_calc/flux_solver.c:187-193). */
enum {
    HYDRO_SOLVER_Q1D = 0,  /* linear_GRP_solver_Edir_Q1D (flux_solver.c:191), the reference's call */
    HYDRO_SOLVER_G2D = 1   /* linear_GRP_solver_Edir_G2D with atc = eps, the alternative the
                              reference keeps commented out at flux_solver.c:189 */
};

typedef struct hydro2d hydro2d_t;

/* Outcome of a run, in the reference's terms. */
typedef struct {
    int k_out;            /* value the reference writes to config[5] */
    int steps_done;       /* time steps whose update was kept */
    int sweeps_launched;  /* kernel launches of the time loop */
    int halted;           /* 0 ran to the end, 1 aborted (last step discarded), 2 stopped after a step */
    int error_code_x;     /* last failing x-face code (0 none, 1 reconstruction, 2 GRP check) */
    int error_code_y;
    double time;          /* final time (time_plot[nt]) */
    double tau;           /* last time step */
    double gpu_ms;        /* device time of the time loop (CUDA events) */
    unsigned long long newton_faces, newton_iters;  /* exact-solver statistics (when enabled) */
    unsigned long long newton_fallbacks;            /* FP32 forms: faces finished by the FP64 iteration */
} hydro_run_info;

/* Create a solver for an m (x) by n (y) grid in the given form. 0 on success. */
int hydro2d_create(hydro2d_t **out, int m, int n, int form);
/* The same with the interface solver chosen (HYDRO_SOLVER_*; hydro2d_create uses
 * HYDRO_SOLVER_Q1D).  HYDRO_SOLVER_G2D is available in HYDRO_FORM_FP64 and
 * HYDRO_FORM_FP32; the learned form is built for the quasi-1D solver (-1). */
int hydro2d_create_ex(hydro2d_t **out, int m, int n, int form, int solver);
void hydro2d_destroy(hydro2d_t *h);
/* Upload an x-major (value of cell (j,i) at [j*n+i]) FP64 state; E may be NULL,
 * then E = 0.5 u^2 + p/(gamma-1)/rho + 0.5 v^2 as the reference's driver computes it. */
int hydro2d_upload(hydro2d_t *h, const double *rho, const double *u, const double *v, const double *p,
                   const double *E, double gamma);
int hydro2d_download(hydro2d_t *h, double *rho, double *u, double *v, double *p, double *E);
/* Run the time loop configured by cfg[0..ncfg) (config[] semantics) from the
 * uploaded state: split = 0 unsplit, 1 dimension split.  stats != 0 counts
 * Newton faces/iterations. */
int hydro2d_run(hydro2d_t *h, const double *cfg, int ncfg, int split, int stats, hydro_run_info *info);
/* 1D run (order 1 = Godunov, 2 = GRP) of an m-cell tube held in host arrays,
 * configured by cfg[] like the 1D scheme entry points, with no plot snapshots.
 * rho, u, p (and E) hold the initial state and receive the final one; E is the
 * initial specific total energy, or NULL to use the 1D driver's formula. */
int hydro1d_run(int m, double *rho, double *u, double *p, double *E, const double *cfg, int ncfg, int order,
                hydro_run_info *info);
/* The Lagrangian schemes the same way; X (m+1 doubles, may be NULL) receives
 * the final node coordinates, which start at j * cfg[10]. */
int hydro1d_run_lag(int m, double *rho, double *u, double *p, double *E, double *X, const double *cfg, int ncfg,
                    int order, hydro_run_info *info);
/* Kernel variants of the unsplit step (tile shape / threads / occupancy).
 * hydro2d_get_variant fills shape[5] = {tile x, tile y, threads, min CTAs per SM,
 * kind}: kind 0 = one CTA per tile, 1 or 2 = the persistent TMA-staged kernel
 * with that many shared-memory stages, 3 = the FP32 strip kernel (tile x = rows
 * per work unit, tile y = columns a strip updates). */
int hydro2d_num_variants(hydro2d_t *h);
int hydro2d_set_variant(hydro2d_t *h, int v);
int hydro2d_get_variant(hydro2d_t *h, int *shape);
/* Autotuner: times every variant on `steps` steps of the uploaded state (which
 * is restored), keeps the fastest and returns its index; times_ms (may be
 * NULL) receives one time per variant. */
int hydro2d_autotune(hydro2d_t *h, const double *cfg, int ncfg, int steps, float *times_ms);
/* Allocation-free 1D run (no counterpart in the reference): for callers that
 * cannot allocate device memory -- frameworks that own the device pool through
 * their own allocator, drivers with a fixed memory budget.  d_state is the
 * caller's device buffer [4][m] (rho, u, p, E), initial state in, final state
 * out; the scheme's scratch is a fixed static device array of the library
 * (20 m + 19 doubles for at most 16384 cells, held by every GPU that loads the
 * library; larger m returns -3 with a message).  The first call on a device
 * looks the array's address up (cached per device); calls share the array, so
 * overlapping calls race and must be serialised.  stream: a cudaStream_t
 * (NULL = legacy default stream).  Nothing is allocated or freed; the call
 * copies its result words to the host and waits for its stream. */
int hydro1d_run_noalloc(int m, double *d_state, const double *cfg, int ncfg, int order, void *stream,
                        hydro_run_info *info);
/* Measured FP64 fused multiply-add rate of the current GPU (DFMA per second,
 * all SMs, no memory traffic): the FP64 pipe's peak for the roofline of the
 * FP64 form (no reference counterpart). */
int hydro_fp64_peak(double *dfma_per_s);
/* ---- learned Newton starting pressure (no reference counterpart) ---------
 * A 6-64-64-1 ReLU network predicting log(p_star / sqrt(pL pR)) of a Riemann problem
 * from scale-free features; trained on the GPU by this library's own
 * forward/backward/Adam kernels on problems labelled by the FP64 exact solver.
 * Parameters are a flat float[4673]: W1[64][6], b1[64], W2[64][64], b2[64],
 * w3[64], b3. */
#define HYDRO_MLP_NPARAM 4673
/* A solver of the learned form installs the trained network shipped with the
 * library when it is created: the file named by $HYDRO_MLP_WEIGHTS, else
 * weights/riemann_guess_6_64_64_1.f32 beside the library's build folder
 * (so GRP_solver_2D_EUL_source with config[300] = 2 needs no extra call). */
typedef struct hydro_mlp hydro_mlp_t;
int hydro_mlp_create(hydro_mlp_t **out, unsigned long long seed);
void hydro_mlp_destroy(hydro_mlp_t *h);
int hydro_mlp_get_params(hydro_mlp_t *h, float *params);
int hydro_mlp_set_params(hydro_mlp_t *h, const float *params);
/* n problems (density/pressure ratios log-uniform in [1e-4,1e4], velocity jump
 * uniform in [-5,5]) generated and labelled on the device; raw_host (may be
 * NULL) receives rhoL,uL,pL,rhoR,uR,pR per problem. */
int hydro_mlp_generate(hydro_mlp_t *h, long long n, unsigned long long seed, double gamma, double *raw_host);
int hydro_mlp_get_data(hydro_mlp_t *h, float *X, float *Y, long long n);
/* Adam with a cosine learning-rate schedule; the last `holdout` problems are
 * not trained on; loss_per_epoch (may be NULL) gets the mean squared error. */
int hydro_mlp_train(hydro_mlp_t *h, int epochs, int batch, float lr, long long holdout, float *loss_per_epoch);
/* Mean squared error and its gradient over n host samples (X[n][6], Y[n]). */
int hydro_mlp_gradient(hydro_mlp_t *h, const float *X, const float *Y, int n, float *grad, float *loss);
/* Tensor-core (BF16 mma) inference on host feature rows. */
int hydro_mlp_predict(hydro_mlp_t *h, const float *X, int n, float *Y);
/* The device feature map of states rhoL,uL,pL,rhoR,uR,pR (rows of 6). */
int hydro_mlp_features(const double *states, int n, double gamma, float *X);
/* Conservation integrals of the current state, summed in FP64 in a fixed
 * order (deterministic): sums[4] = h_x h_y * sum of rho, rho u, rho v, rho E. */
int hydro2d_conservation(hydro2d_t *h, double hx, double hy, double *sums);
/* Install network parameters into a solver of the HYDRO_FORM_FP32_LEARNED form. */
int hydro2d_set_mlp(hydro2d_t *h, const float *params);
/* What the learned start costs and saves in the FP32 form's device code, on
 * nfaces (rounded down to a multiple of 32, at least 32) seeded Riemann pairs
 * with the four-quadrant data's ranges, all through the exact path, one thread
 * per face.  out[10]: ns per face of the network (features + three BF16 MMA
 * layers); of the exact solve from the reference's start (half the tangent
 * intersection); its mean Newton iterations; of the exact solve from the
 * network's start (network excluded); its mean iterations; ns per FP32 Newton
 * iteration (the solves' difference over the iterations saved); ns per face of
 * the nonlinear GRP derivatives and fluxes after the solve; of the whole exact
 * face from the reference's start; of the exact solve from the FP32 form's own
 * start (the tangent intersection); its mean iterations. */
int hydro_learned_costs(const float *params, int nfaces, unsigned long long seed, double gamma, double *out);
/* ---- batched problems (no reference counterpart) --------------------------
 * Many independent 2D unsplit GRP problems of uneven grid size m x n on the
 * unit square (h_x = 1/m, h_y = 1/n) advanced together for a fixed number of
 * steps in the FP32 form.  Each problem has its own CFL time step from its own
 * initial data (as grp_solver_2D_EUL_source.c:180-200 does for one grid) and
 * its own halting; its result equals a one-problem FP32 run of that grid.
 * config[] supplies gamma, eps, CFL, alpha and the boundary codes (17, 18) for
 * all problems; t_all is ignored.
 * Schedules: 0/1 persistent cooperative kernel, static tiles (problem-major /
 * largest problem first), 2/3 the same with a dynamic tile counter, 4 a CUDA
 * graph of one launch per step.  Shapes: tiles of the one-grid tile kernel, or
 * strip units (60 columns x a run of rows) of the one-grid strip kernel.  The persistent kernel separates the steps
 * with a grid barrier whose wait is limited (default 5 s,
 * hydro_batch_set_wait_limit); a wait that runs out makes the run return -2. */
typedef struct hydro_batch hydro_batch_t;
typedef struct {
    double gpu_ms;            /* device time of the time loop */
    int shape, schedule;      /* tile shape index and schedule used */
    int graphed;              /* 1 if the time loop ran as one captured CUDA graph */
    int steps, tiles;         /* steps run; tiles per step over all problems */
    int halted_problems;      /* problems that stopped or aborted early */
    unsigned long long newton_faces, newton_iters, newton_fallbacks; /* with stats = 1 */
} hydro_batch_info;
int hydro_batch_create(hydro_batch_t **out, int nprob, const int *m, const int *n);
void hydro_batch_destroy(hydro_batch_t *b);
/* x-major planes of problem p (E may be NULL: computed as the 2D driver does). */
int hydro_batch_upload(hydro_batch_t *b, int p, const double *rho, const double *u, const double *v, const double *pr,
                       const double *E, double gamma);
int hydro_batch_download(hydro_batch_t *b, int p, double *rho, double *u, double *v, double *pr, double *E);
int hydro_batch_run(hydro_batch_t *b, const double *cfg, int ncfg, int steps, int stats, hydro_batch_info *info);
int hydro_batch_num_shapes(void);
int hydro_batch_num_schedules(void);
/* out4 = {tile cells along y, along x, threads, min CTAs per SM}; for a strip
 * shape {columns a strip updates, rows per work unit, threads, min CTAs per SM} */
int hydro_batch_shape(int shape, int *out4);
/* 0: tiles (the one-grid tile kernel's code), 1: strips (the one-grid strip
 * kernel's per-unit march; at most 576 problems). */
int hydro_batch_shape_kind(int shape);
int hydro_batch_set_schedule(hydro_batch_t *b, int shape, int schedule);
int hydro_batch_set_wait_limit(hydro_batch_t *b, double seconds);
/* Times every (shape, schedule) pair on `steps` steps of the uploaded states
 * (restored afterwards), keeps the fastest and returns shape * schedules +
 * schedule; times_ms (may be NULL) receives shapes x schedules values.  The
 * strip shapes are not timed (3e38): their first steps do not predict a long
 * run; hydro_batch_set_schedule selects them. */
int hydro_batch_autotune(hydro_batch_t *b, const double *cfg, int ncfg, int steps, float *times_ms);
/* Outcome of problem p in the last run: halted (0 no, 1 abort, 2 stop), the
 * step it halted on, and its time step. */
int hydro_batch_problem_info(hydro_batch_t *b, int p, int *halted, int *halted_step, double *tau);

/* One-call form: create, upload, (autotune), run, download, destroy. */
typedef struct {
    int m, n;                 /* grid size */
    double *rho, *u, *v, *p;  /* x-major [m][n]: initial state in, final state out */
    double *E;                /* may be NULL on input (computed) -- then not written */
    int halted, halted_step;  /* out */
    double tau;               /* out: the problem's time step */
} hydro_problem;
typedef struct {
    const double *cfg;        /* config[] */
    int ncfg;
    int autotune_steps;       /* > 0: autotune on that many steps first */
    int shape, schedule;      /* used when not autotuning */
    int stats;
    hydro_batch_info info;    /* out */
} hydro_batch_opts;
int hydro_gb300_batch_run(hydro_problem *probs, int nprob, int steps, hydro_batch_opts *o);

/* ---- two-component interface flux (MULTIFLUID_BASICS) --------------------
 * Replaces GRP_2D_flux of the reference's two-component build
 * (src/flux_calc/flux_solver.c:158-237 with MULTIFLUID_BASICS; struct i_f_var,
 * src/include/var_struc.h:116-142) for a batch of nface independent faces.
 * in:  [40][nface] host array, field k of face f at in[k*nface + f]:
 *      0 n_x, 1 n_y; left side from 2, right side from 21, each 19 fields:
 *      gamma, RHO, U, V, P, d_rho, d_u, d_v, d_p, t_rho, t_u, t_v, t_p,
 *      Z_a, d_z_a, t_z_a, PHI, d_phi, t_phi.
 * out: [18][nface]: F_rho, F_u, F_v, F_e, RHO_int, U_int, V_int, P_int, F_phi,
 *      F_gamma, F_e_a, PHI, Z_a, U_qt_add_c, V_qt_add_c, U_qt_star, V_qt_star, P_star
 *      (the members GRP_2D_flux writes into the left struct).
 * status: [nface] GRP_2D_flux's return value (star_dire_check: 1 non-positive
 *      density or pressure, 2 non-finite t-axis value, 3 non-finite derivative).
 *      Unlike the reference, which returns before writing the fluxes of such
 *      a face, the outputs are written for every face.
 * cfg: the reference's config[] (4 eps, 6 gamma of fluid a, 60 store F_gamma,
 *      106 gamma of fluid b; entries at or beyond ncfg read as INFINITY, the
 *      reference's default).  tau: the time step.
 * Returns 0, -1 on a CUDA error, -2 on bad arguments. */
typedef struct {
    int n_bad;          /* faces with a non-zero status */
    int first_bad;      /* smallest such face index, -1 if none */
    int first_code;     /* its status */
    int resumed[4];     /* faces taken up by the 2nd..5th pass (the 1st completes the uniform pairs and
                           queues the rest; each later one stops at an iteration cap) */
    double kernel_ms;   /* device time of the flux kernels */
} hydro_face_info;
int hydro_grp2d_flux_mf(int nface, const double *in, double *out, int *status, const double *cfg, int ncfg,
                        double tau, hydro_face_info *info);

/* The FP64 form's uniform-pair threshold (host arithmetic, no GPU): the largest
   d2 whose correctly rounded square root is below eps (-1 if none), so that the
   reference's test sqrt(d2) < eps (linear_grp_solver_Edir_Q1D.c:95-96,139,
   linear_grp_solver_Edir_G2D.c:112-113,156, with atc = eps) is decided as
   d2 <= this value. */
double hydro_uniform_dist2_max(double eps);

/* The 2D scheme entry points (GRP_solver_2D_[split_]EUL_source) keep the last
   call's solver -- its device buffers, kernel set-up and network -- for the
   next call with the same grid, form and interface solver (environment
   HYDRO_SOLVER_CACHE=0: no solver is kept).  This frees the kept solver. */
void hydro_gb300_release_cache(void);

/* Number of CUDA kernels launched by this library since load (all solvers). */
unsigned long long hydro_gb300_kernel_launches(void);
/* Message of the last failing call in this thread ("" if none). */
const char *hydro_gb300_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
