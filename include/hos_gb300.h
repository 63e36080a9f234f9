/*
 * hos_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the high-order-solver 2D
 * per-step hot path: WENO5/7/9-AO reconstruction with the discontinuity-feedback factor,
 * the second-order gas-kinetic (GKS) flux, the two-stage fourth-order (S2O4) update, the
 * ghost-cell fill and the CFL time-step reduction.
 *
 * Plain C types only (pointers, sizes, doubles); no CUDA or C++ types cross this boundary.
 * Every function returns an int status: 0 ok, HOS_E_* otherwise.  Nothing calls exit().
 *
 * Reference interface replaced (XJTUZhangHong/high-order-solver, file:line):
 *   problem setup globals + Block2d + allocators ... src/2Dproblem.cpp:7-81,
 *        include/fluid_mesh.h:82-222, src/basic_function.cpp:1310-1491   -> hos2d_create
 *   Fluid2d::convar / primvar of the initial data .... src/2Dproblem.cpp:345-385 -> hos2d_set_state
 *   reading Fluid2d arrays back (output2d) ............ src/output.cpp:64-84     -> hos2d_get_state
 *   CopyFluid_new_to_old + Get_CFL ..................... src/basic_function.cpp:1571-1584,
 *                                                        src/time_advance.cpp:264-305 -> hos2d_begin_step
 *   the four BoundaryCondition2d calls ................. src/boundary_condition.cpp:66-442 -> hos2d_boundary
 *   one stage: BCs, Convar_to_Primvar, Reconstruction_within_cell, Reconstruction_forg0,
 *     Calculate_flux, Update, Update_alpha ............. src/2Dproblem.cpp:137-157  -> hos2d_stage
 *   one time step (the body of the driver's while loop) src/2Dproblem.cpp:128-159  -> hos2d_step
 */
#ifndef HOS_GB300_H
#define HOS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define HOS_OK 0
#define HOS_E_BLOWUP 1      /* negative density/pressure or NaN: where the reference exits */
#define HOS_E_CONFIG 2      /* unsupported or inconsistent parameters                    */
#define HOS_E_CUDA 3        /* CUDA runtime error (no device, launch failure, ...)       */
#define HOS_E_ARG 4         /* null pointer or bad argument                              */
#define HOS_E_NOMEM 5       /* device allocation failed                                  */
#define HOS_E_TIMEOUT 6     /* a device-side wait (TMA tile load) ran past its limit      */

/* boundary kinds, per side (left, right, down, up) */
#define HOS_BC_FREE 0       /* free_boundary_*  (zero-gradient outflow)  */
#define HOS_BC_PERIODIC 1   /* periodic_boundary_*                       */
#define HOS_BC_REFLECT 2    /* reflection_boundary_*                     */
#define HOS_BC_INFLOW 3     /* inflow_boundary_* with a fixed primitive state */
/* the reference's double-Mach-reflection boundary (boundaryforDoubleMach,
 * src/2Dproblem.cpp:1029-1093): an oblique shock hitting a wedge wall that starts at
 * x = wedge_x0; the left side must be HOS_BC_INFLOW with the post-shock state */
#define HOS_BC_WEDGE_BOTTOM 4 /* bottom: post-shock state for x < x0, reflecting wall after */
#define HOS_BC_WEDGE_TOP 5    /* top: post-shock state left of the moving shock, pre-shock right */
#define HOS_BC_NOSLIP 6       /* noslip_adiabatic_boundary_*: mirrored density and energy, momentum
                                 2 rho u_wall - rho u (both components); wall velocity
                                 (bc_prim[side][1], bc_prim[side][2]) */

/* time-marching methods (the reference's TimeMarchingCoefficient_2d slot values) */
#define HOS_INT_S2O4 0      /* two-stage fourth order (default)           */
#define HOS_INT_S1O1 1      /* one stage, first order                     */
#define HOS_INT_S1O2 2      /* one stage, second order (flux time derivative) */
#define HOS_INT_RK2 3       /* two-stage Runge-Kutta                      */
#define HOS_INT_RK3 4       /* three-stage strong-stability-preserving RK */
#define HOS_INT_RK4 5       /* classical four-stage Runge-Kutta           */
/* interface fluxes (the reference's Flux_function_2d slot values) */
#define HOS_FLUX_GKS 0      /* GKS2D, second order                        */
#define HOS_FLUX_LF 1       /* LF2D, Lax-Friedrichs (Euler)               */

/* compute precision of reconstruction and flux; state, stage combination and the CFL
 * reduction are FP64 in both */
#define HOS_FP64 0
#define HOS_FP32 1

/* Problem parameters: the globals and Block2d fields a reference 2D driver sets
 * (src/2Dproblem.cpp:7-81).  Gausspoint must match the order: 5 -> 2, 7 -> 3, 9 -> 4. */
typedef struct hos_params2d {
    int nodex, nodey;       /* interior cells (Block2d::nodex / nodey)          */
    int ghost;              /* ghost layers (Block2d::ghost), >= order/2 + 1    */
    int order;              /* WENO-AO order: 5, 7 or 9                         */
    int gausspoint;         /* Gauss points per face                           */
    int characteristic;     /* reconstruction_variable: 1 characteristic, 0 conservative */
    int use_df;             /* is_using_df_factor: 1 the DF variants (WENO5/7/9), 0 the
                               non-DF WENO5-AO the drivers install first (order 5, 2 Gauss
                               points; WENO5_AO_normal / WENO5_AO_tangent) */
    int K;                  /* internal degrees of freedom                      */
    double gamma;           /* Gamma                                            */
    double c1_euler, c2_euler; /* numerical collision time tau_num = c1 dt + c2 dt |dp|/|p| */
    double cfl;             /* Block2d::CFL                                     */
    double left, right, down, up;  /* domain                                   */
    int bc[4];              /* HOS_BC_* for left, right, down, up               */
    double bc_prim[4][4];   /* inflow primitive state (rho, u, v, p) per side   */
    /* wedge boundaries (HOS_BC_WEDGE_*): wall start, speed of the shock's trace along the
     * top (20/sqrt(3) for the reference's Mach 10), post- and pre-shock primitive states */
    double wedge_x0;
    double wedge_top_speed;
    double wedge_post[4];
    double wedge_pre[4];
    /* time marching (timecoe_list_2d, src/time_advance.cpp:197-247) and flux
     * (flux_function_2d, src/flux_function.cpp:314-754); 0 / 0 = S2O4 with GKS2D */
    int integrator;         /* HOS_INT_*  */
    int flux;               /* HOS_FLUX_* */
    /* collision time (tau_type, src/basic_function.cpp:638-708): HOS_TAU_EULER, or
     * HOS_TAU_NS with the physical tau = 2 Mu lambda / rho (or 2 Nu lambda) added to the
     * numerical one, and the viscous time-step cap of Dtx (src/time_advance.cpp:292-305);
     * prandtl_fix = is_Prandtl_fix, with Prandtl number prandtl (= Pr) */
    int tau_type;
    double mu, nu;
    int prandtl_fix;
    double prandtl;
    /* nonlinear weights of the non-DF WENO5-AO scheme (use_df = 0; the reference's wenotype
     * global, src/reconstruction.cpp:7): HOS_WENO_Z, HOS_WENO_JS or HOS_WENO_LINEAR */
    int wenotype;
} hos_params2d;

/* wenotype values (WENOtype, include/reconstruction.h in the reference: linear, wenojs,
 * wenoz); zero is the Z-type weights every reference 2D driver selects */
#define HOS_WENO_Z 0
#define HOS_WENO_JS 1
#define HOS_WENO_LINEAR 2

#define HOS_TAU_EULER 0
#define HOS_TAU_NS 1

typedef struct hos_solver2d hos_solver2d;

/* Allocate the device state for one problem on the current CUDA device. */
int hos2d_create(const hos_params2d* params, int precision, hos_solver2d** out);
int hos2d_destroy(hos_solver2d* s);

/* Block sizes: nx = nodex + 2 ghost, ny = nodey + 2 ghost; state arrays hold nx*ny cells,
 * cell (i, j) at i*ny + j, 4 doubles per cell (the reference's Fluid2d order). */
int hos2d_dims(const hos_solver2d* s, int* nx, int* ny);

/* Upload the conserved state (host, [nx*ny][4]) and optionally the primitive state the
 * first step's CFL reads (host, [nx*ny][4], may be NULL: then derived from convar).
 * Resets time to 0 and the DF indicators to 0.  Synchronous.  Pinned host buffers
 * (cudaHostAlloc, cudaMallocHost, cudaHostRegister) are read by the upload kernel over the host
 * link; other host memory goes through a device staging copy first. */
int hos2d_set_state(hos_solver2d* s, const double* convar, const double* primvar);
/* Same from device memory already resident in HBM (SoA planes [4][nx*ny]). */
int hos2d_set_state_device(hos_solver2d* s, const double* d_convar_soa, const double* d_primvar_soa);

/* Restore the DF indicators alpha_x, alpha_y (host, [nx*ny]) of a state captured mid-run
 * (Fluid2d::alpha_x / alpha_y, include/fluid_mesh.h:146-147).  Synchronous. */
int hos2d_set_alpha(hos_solver2d* s, const double* alpha_x, const double* alpha_y);

/* Download the conserved state, its primitive variables, alpha_x, alpha_y (host arrays;
 * any pointer may be NULL).  Synchronous.  Pinned convar / primvar buffers are written by the
 * transposition kernel over the host link; other host memory through a device staging copy. */
int hos2d_get_state(hos_solver2d* s, double* convar, double* primvar, double* alpha_x, double* alpha_y);

/* Replace the four boundary kinds (HOS_BC_*, left, right, down, up) and, when bc_prim is not
 * NULL, the inflow primitive states ([4][4], same order): the driver reassigning its
 * BoundaryCondition2d slots (src/2Dproblem.cpp:20-28).  Waits for queued work. */
int hos2d_set_boundary(hos_solver2d* s, const int* bc, const double* bc_prim);
/* Set the simulation time (Block2d::t) the next step starts from.  Synchronous. */
int hos2d_set_time(hos_solver2d* s, double t);
/* Reconstruction of the following stages: HOS_RECON_WENO (the WENO-AO-DF scheme of the
 * solver's order, the default) or HOS_RECON_FIRST_ORDER (First_order_normal /
 * First_order_tangent, src/reconstruction.cpp:1537-1560, 2214-2231: cell averages, zero
 * slopes -- the step-0 scheme of the reference's drivers when is_using_df_factor is set,
 * e.g. src/2Dproblem.cpp:733-745).  The Gauss points stay those of the solver's order. */
#define HOS_RECON_WENO 0
#define HOS_RECON_FIRST_ORDER 1
int hos2d_set_reconstruction(hos_solver2d* s, int mode);
/* 1: the stage update is Update_with_source (src/time_advance.cpp:534-704, the RT_instability
 * driver): gravity source S = (0, 0, rho, rho v); under S2O4 stage 0 sets
 * W = W_old + dt (L(W) + S(W)) from the stage's Gauss-weighted fluxes f and stage 1 leaves the
 * state (fluxes and DF indicators are still computed), as the reference does.  S2O4 only. */
int hos2d_set_source(hos_solver2d* s, int on);

/* CopyFluid_new_to_old + Get_CFL: fix this step's dt (clipped to tstop). Asynchronous. */
int hos2d_begin_step(hos_solver2d* s, double tstop);
/* Ghost-cell fill of the current state (the wedge boundary at the current step's start
 * time). Asynchronous. */
int hos2d_boundary(hos_solver2d* s);
/* One S2O4 stage (0 or 1) with the dt fixed by hos2d_begin_step. Asynchronous. */
int hos2d_stage(hos_solver2d* s, int stage);
/* One full time step (begin_step + two stages). Asynchronous. */
int hos2d_step(hos_solver2d* s, double tstop);
/* nsteps full steps; replays a captured CUDA graph of one step when use_graph != 0. */
int hos2d_advance(hos_solver2d* s, int nsteps, double tstop, int use_graph);

/* Wait for queued work; report time, last dt and the blow-up status (HOS_E_BLOWUP). */
int hos2d_sync(hos_solver2d* s, double* t, double* dt);

/* One full time step with CUDA events between its launches; synchronises and writes the
 * device time in milliseconds of each launch, in order: begin_step, then per stage
 * bc_fill, gate (0 without a gate), x-face kernel, y-face kernel, update (11 values).  The reference has no
 * counterpart; it replaces its clock()-based Runtime timer (include/output.h:15-25) with
 * per-kernel device timing. */
int hos2d_profile_step(hos_solver2d* s, double tstop, double* ms);

/* Number of kernel launches one hos2d_step enqueues. */
int hos2d_launches_per_step(const hos_solver2d* s);

/* The CUDA stream the solver enqueues on (as an opaque pointer, for event timing). */
void* hos2d_stream(hos_solver2d* s);

/* Human-readable text of the last error on this thread. */
const char* hos_last_error(void);

/* Self-test of the device-side wait limit (no counterpart in the reference): one block waits
 * on an mbarrier that nothing completes, with the bounded wait the TMA tile loads and the
 * gate's tensor-core MMAs use.  Returns HOS_E_TIMEOUT when the wait gave up as designed (after
 * about a second) and the context is still usable, HOS_OK if the wait had completed (a fault
 * in the limit), HOS_E_CUDA on a launch error. */
int hos_wait_limit_selftest(void);

/* Self-test of the FP32 -> FP64 conversion the FP32 face kernels' stage combination runs on the
 * integer pipes (no counterpart in the reference): y[i] = x[i] widened on the device, n host
 * values.  Exact for normal values and zero; FP32 subnormals give signed zero. */
int hos_convert_selftest(const float* x, double* y, size_t n);

/* ---- learned gate (FP32-bulk path; no counterpart in the reference) ---------------------
 * A 16 -> 32 -> 32 -> 1 MLP (BF16 weights, FP32 accumulation on the tensor cores) predicts,
 * per cell and direction, from the normalised WENO-AO smoothness indicators of density and
 * pressure and the DF indicator, whether the nonlinear weights of all characteristic variables
 * stay within 0.02 of the linear weights; predicted-smooth cells reconstruct with the
 * full-stencil polynomial, everything else (and every linear result failing the positivity /
 * oscillation check) with full WENO-AO.  Labels come from the solver's own states
 * (hos_gate_collect); training runs on the GPU (hos_gate_train). */
#define HOS_GATE_FEATURES 16
#define HOS_GATE_SAMPLE 20     /* floats per sample: 16 features, label (1 smooth), distance, cell, direction */
#define HOS_GATE_PARAMS 1633   /* W1[32][16] b1[32] W2[32][32] b2[32] w3[32] b3 */
typedef struct hos_gate hos_gate;
int hos_gate_create(unsigned long long sample_capacity, unsigned seed, hos_gate** out);
int hos_gate_destroy(hos_gate* g);
int hos_gate_get_params(hos_gate* g, float* params);
int hos_gate_set_params(hos_gate* g, const float* params);
/* append labelled samples of a solver's current state: cells whose hash has sample_log2 low
 * zero bits, both directions */
int hos_gate_collect(hos_gate* g, hos_solver2d* s, int sample_log2);
int hos_gate_sample_count(hos_gate* g, unsigned long long* n);
int hos_gate_get_samples(hos_gate* g, float* out, unsigned long long n);
int hos_gate_set_samples(hos_gate* g, const float* in, unsigned long long n);
int hos_gate_clear_samples(hos_gate* g);
/* gradient (HOS_GATE_PARAMS floats) and loss of the class-weighted mean cross-entropy over
 * samples [first, first + n); no parameter update */
int hos_gate_gradient(hos_gate* g, unsigned long long first, int n, float w_pos, float w_neg, float* grad,
                      double* loss);
int hos_gate_forward(hos_gate* g, unsigned long long first, int n, float* logits);
/* steps Adam updates on mini-batches of batch samples */
int hos_gate_train(hos_gate* g, int steps, int batch, float lr, float w_pos, float w_neg, unsigned seed,
                   double* mean_loss);
const char* hos_gate_last_error(void);
/* attach a copy of the network to an FP32 solver (NULL detaches): cells with logit above
 * threshold take the linear path; predicted-smooth cells whose hash has audit_log2 low zero
 * bits are re-checked with full weights */
int hos2d_set_gate(hos_solver2d* s, const hos_gate* g, float threshold, int audit_log2);
/* a-posteriori check of the linear path: a linear reconstruction is kept when its density and
 * total energy lie within the three central cells' range widened by slack times that range
 * (default 0.1; 0 accepts only values inside the range) and its temperature is positive;
 * otherwise the full WENO-AO reconstruction replaces it.  No counterpart in the reference. */
int hos2d_set_gate_check(hos_solver2d* s, double slack);
/* reuse != 0: the network runs at the first stage of each step only; the later stages take its
 * flags dilated by one cell along each flag's axis (a cell keeps its x / y flag when both its
 * x / y neighbours have it), which covers the at most quarter-cell motion of a front within a
 * stage.  0 (the default): the network runs at every stage.  No counterpart in the reference. */
int hos2d_set_gate_reuse(hos_solver2d* s, int reuse);
/* counters since the last reset: cells gated x, y; predicted smooth x, y; audited; audited but
 * not smooth (false negatives of the gate); linear results rejected; (unused) */
int hos2d_gate_stats(hos_solver2d* s, unsigned long long* stats, int reset);
/* what the a-posteriori check did with the gate's errors: out[0] linear reconstructions in
 * cell-directions an audit found not smooth (predicted smooth, full weights farther than the
 * label's tolerance from the linear ones), out[1] how many of them the check accepted (the rest
 * fell back to WENO-AO); counted at the stages where the network runs, reset with
 * hos2d_gate_stats.  No counterpart in the reference. */
int hos2d_gate_audit_check(hos_solver2d* s, unsigned long long* out);

/* ---- 1D path --------------------------------------------------------------------------
 * The reference's 1D drivers (SodTubeProblem, accuracy_sinwave_1d, src/1Dproblem.cpp:3-149,
 * 519-735) over Fluid1d arrays: state of cell i at index i over the full line including
 * ghosts, 3 doubles per cell (rho, rho*u, rho*E).  Replaces (file:line):
 *   globals + Block1d + SetUniformMesh ..... src/1Dproblem.cpp:8-76            -> hos1d_create
 *   ICforSodTube / ICfor_sinwave ........... src/1Dproblem.cpp:151-174, 692-706 -> hos1d_set_state
 *   output1d ............................... src/output.cpp:3-15               -> hos1d_get_state
 *   loop body: CopyFluid_new_to_old, Get_CFL, boundaries, Reconstruction_within_cell,
 *     Reconstruction_forg0, Calculate_flux, Update, Update_alpha (src/1Dproblem.cpp:93-131)
 *                                                                               -> hos1d_step
 *   the while loop to tstop ................ src/1Dproblem.cpp:78-148          -> hos1d_run */
typedef struct hos_params1d {
    int nodex, ghost;
    int order;            /* 5, 7, 9                                                        */
    int characteristic;   /* reconstruction_variable                                        */
    int df_mode;          /* 0: WENO5-AO (no DF) every step; 1: DF variant every step;
                             2: WENO5-AO at step 0, then WENO5-AO-DF (the Sod driver)         */
    int update_alpha;     /* 1: Update_alpha after every stage (Sod); 0: never (accuracy)  */
    int K;
    double gamma;
    double c1_euler, c2_euler;
    double cfl;
    double left, right;
    int bc[2];            /* HOS_BC_FREE, HOS_BC_PERIODIC or HOS_BC_REFLECT, left and right */
    int wenotype;         /* weights of the non-DF WENO5-AO steps: HOS_WENO_Z, _JS or _LINEAR */
} hos_params1d;

typedef struct hos_solver1d hos_solver1d;

int hos1d_create(const hos_params1d* params, int precision, hos_solver1d** out);
int hos1d_destroy(hos_solver1d* s);
/* host arrays [nx][3]; set_state resets time, step count and DF indicators (synchronous) */
int hos1d_set_state(hos_solver1d* s, const double* convar);
int hos1d_get_state(hos_solver1d* s, double* convar, double* alpha);
/* one S2O4 step (asynchronous); steps queued once t >= tstop do nothing */
int hos1d_step(hos_solver1d* s, double tstop);
/* steps until t >= tstop or max_steps more steps; steps_done (may be NULL) receives the
 * number of steps taken since hos1d_set_state */
int hos1d_run(hos_solver1d* s, double tstop, int max_steps, int* steps_done);
int hos1d_sync(hos_solver1d* s, double* t, double* dt);
/* The step in pieces, for callers that keep the reference's loop (src/1Dproblem.cpp:96-131):
 * begin_step = CopyFluid_new_to_old + Get_CFL (dt then readable through hos1d_sync), stage =
 * boundaries + reconstruction + flux + Update + Update_alpha of S2O4 stage 0 or 1.  Both are
 * asynchronous. */
int hos1d_begin_step(hos_solver1d* s, double tstop);
int hos1d_stage(hos_solver1d* s, int stage);
/* Replace the two boundary kinds (the driver reassigning its BoundaryCondition slots). */
int hos1d_set_boundary(hos_solver1d* s, const int* bc);
/* Restore the DF indicators (Fluid1d::alpha, host [nx]) and the simulation time. */
int hos1d_set_alpha(hos_solver1d* s, const double* alpha);
int hos1d_set_time(hos_solver1d* s, double t);
const char* hos1d_last_error(void);

/* ---- 3D path --------------------------------------------------------------------------
 * The reference's 3D driver (CubicTube, src/3Dproblem.cpp:3-172): non-DF WENO5-AO face values,
 * tangential sweeps to 2 x 2 Gauss points per face (gausspoint = 4, weights 1/4), GKS3D, S2O4,
 * over Fluid3d arrays: state of cell (i, j, k) at (i*ny + j)*nz + k over the full block
 * including ghosts, 5 doubles per cell (rho, rho u, rho v, rho w, rho E).  Replaces (file:line):
 *   globals + Block3d + SetUniformMesh ..... src/3Dproblem.cpp:8-97           -> hos3d_create
 *   ICfor_cubic_sod (any initial state) .... src/3Dproblem.cpp:174-219         -> hos3d_set_state
 *   output3d ............................... src/output.cpp                    -> hos3d_get_state
 *   loop body: CopyFluid_new_to_old, Get_CFL, six boundaries, Convar_to_primvar,
 *     Reconstruction_within_cell, Reconstruction_forg0, Calculate_flux, Update_gauss
 *     (src/3Dproblem.cpp:125-157) ........................................... -> hos3d_step
 * GKS3D there converts the face states with Convar_to_primvar_3D and uses the pressure where the
 * Maxwellian's lambda belongs (src/flux_function.cpp:831-836); this library uses lambda, as the
 * reference's 1D and 2D fluxes do.  Sides may be free (the reference's only 3D boundary),
 * periodic or reflecting; tau_type 1 adds the Navier-Stokes collision time 2 mu lambda / rho
 * (Get_Tau_NS / Get_Tau, src/basic_function.cpp:638-708) and the viscous time-step cap of Dtx_3d
 * (src/time_advance.cpp:826-848). */
typedef struct hos_params3d {
    int nodex, nodey, nodez, ghost;   /* ghost >= 3                                      */
    int characteristic;               /* reconstruction_variable                         */
    int K;                            /* internal degrees of freedom (2 for gamma 1.4)   */
    double gamma;
    double c1_euler, c2_euler;
    double cfl;
    int tau_type;                     /* 0 Euler, 1 Navier-Stokes                        */
    double mu;                        /* dynamic viscosity (tau_type 1)                   */
    double left, right, down, up, back, front;
    int bc[6];                        /* left, right, down, up, back, front: HOS_BC_FREE,
                                         HOS_BC_PERIODIC or HOS_BC_REFLECT                */
    int prandtl_fix;                  /* 1: Prandtl-number correction of the heat flux    */
    double prandtl;                   /* Pr (prandtl_fix = 1)                             */
    /* 1 (FP64 only, no Prandtl fix): the reference's own GKS3D convention, which hands
     * Convar_to_primvar_3D's pressure to every slot where lambda belongs (the Maxwellian
     * moments, micro-slopes and collision times, src/flux_function.cpp:831-836, 914), to
     * compare with outputs of the reference's 3D code; 0 (default): lambda, as 1D and 2D do */
    int gks3d_pressure_slot;
} hos_params3d;

typedef struct hos_solver3d hos_solver3d;

/* precision HOS_FP64, or HOS_FP32 for the reconstruction and flux (state, stage combination
 * and CFL stay FP64) */
int hos3d_create(const hos_params3d* params, int precision, hos_solver3d** out);
int hos3d_destroy(hos_solver3d* s);
/* host arrays [ncell][5]; primvar (may be NULL) gives the primitives the first Get_CFL reads
 * (rho, u, v, w, p); otherwise they are converted from convar.  Synchronous. */
int hos3d_set_state(hos_solver3d* s, const double* convar, const double* primvar);
/* convar and/or primvar (either may be NULL), [ncell][5]; synchronous */
int hos3d_get_state(hos_solver3d* s, double* convar, double* primvar);
/* one S2O4 step (asynchronous); steps queued once t >= tstop do nothing */
int hos3d_step(hos_solver3d* s, double tstop);
int hos3d_advance(hos_solver3d* s, int nsteps, double tstop);
int hos3d_sync(hos_solver3d* s, double* t, double* dt);
/* the step in pieces, as the reference's loop calls it */
int hos3d_begin_step(hos_solver3d* s, double tstop);
int hos3d_stage(hos_solver3d* s, int stage);
int hos3d_set_time(hos_solver3d* s, double t);
/* the solver's CUDA stream (cudaStream_t) */
int hos3d_stream(hos_solver3d* s, void** stream);
/* one step with an event after every launch: ms[0] begin, then per stage (12 each):
 * boundaries, gate (0 without one), face/line/point+flux of x, of y, of z, update; n >= 25 */
int hos3d_profile_step(hos_solver3d* s, double tstop, float* ms, int n);
/* The learned gate on the 3D FP32-bulk path (the 2D gate's network and training; inputs are
 * the WENO5-AO indicators of each cell's stencil along x, y and z): predicted-smooth
 * reconstructions along an axis take the big-stencil polynomial in conservative variables,
 * checked a posteriori.  g == NULL detaches.  The solver copies the network. */
int hos3d_set_gate(hos_solver3d* s, const hos_gate* g, float threshold, int audit_log2);
/* counters since the last reset: cells gated along x, y, z; predicted smooth along x, y, z;
 * audited; audited but not smooth; linear results rejected; (unused) */
int hos3d_gate_stats(hos_solver3d* s, unsigned long long* stats, int reset);
/* training samples from a 3D solver's current state (boundaries filled first) */
int hos_gate_collect3d(hos_gate* g, hos_solver3d* s, int sample_log2);
const char* hos3d_last_error(void);

/* ---- batches of independent 2D problems ------------------------------------------------
 * No counterpart in the reference (each of its drivers advances one Block2d).  count
 * problems of uneven sizes, one stop time each, advanced together: one launch per phase for
 * the whole batch (face kernels persist over a table of every problem's tiles), each problem
 * keeping its own dt, boundaries and stop time; problems that reach their stop time idle.
 * All problems share the WENO-AO order and the precision.  Per problem the operations are
 * those of hos2d_step, so results equal the single-problem solver's. */
typedef struct hos_batch2d hos_batch2d;
int hos_batch2d_create(const hos_params2d* params, const double* tstop, int count, int precision,
                       hos_batch2d** out);
int hos_batch2d_destroy(hos_batch2d* b);
int hos_batch2d_set_state(hos_batch2d* b, int k, const double* convar, const double* primvar);
int hos_batch2d_get_state(hos_batch2d* b, int k, double* convar, double* alpha_x, double* alpha_y);
/* time each face-tile shape (reps launches) on the current state and keep the fastest per
 * direction; chosen[2] receives the shape indices, ms[6] the times (either may be NULL) */
int hos_batch2d_autotune(hos_batch2d* b, int reps, int* chosen, double* ms);
/* nsteps batch steps; with use_graph the step is captured once and replayed */
int hos_batch2d_advance(hos_batch2d* b, int nsteps, int use_graph);
/* problems still running, per-problem time, the batch step index of each problem's last step
 * and per-problem failure flags (arrays of count, may be NULL).  A problem whose state turns
 * bad (negative density/pressure or NaN: the reference's exit) stops stepping; the others go
 * on.  With failed == NULL such a failure is reported as HOS_E_BLOWUP. */
int hos_batch2d_status(hos_batch2d* b, int* active, double* t, int* last_step, int* failed);
/* reconstruction of the following steps of every problem: HOS_RECON_WENO or
 * HOS_RECON_FIRST_ORDER (the drivers' first-order step 0, as hos2d_set_reconstruction);
 * waits for queued work */
int hos_batch2d_set_reconstruction(hos_batch2d* b, int mode);
/* attach a copy of a learned gate to an FP32 batch (NULL detaches); counters as hos2d_gate_stats */
int hos_batch2d_set_gate(hos_batch2d* b, const hos_gate* g, float threshold, int audit_log2);
int hos_batch2d_gate_stats(hos_batch2d* b, unsigned long long* stats, int reset);
long long hos_batch2d_cells(const hos_batch2d* b);
void* hos_batch2d_stream(hos_batch2d* b);
const char* hos_batch2d_last_error(void);

/* ---- allocation-free step ------------------------------------------------------------
 * No counterpart in the reference.  For callers that may not allocate device memory once
 * running (a code that reserves its whole HBM budget in its own pool at start-up, or runs
 * under a fixed memory quota on a shared GPU): one S2O4 step on caller-owned device
 * buffers, with the step's scratch in a fixed static device array (about 11.7 MB, held by
 * every GPU that loads the library until exit) and no cudaMalloc / cudaFree.
 *   d_W        conserved state, SoA planes [4][nx*ny], ghosts included (in/out)
 *   d_alpha_x, d_alpha_y   DF indicators [nx*ny] (in/out; zero before the first step)
 *   dt         the step's time step (the caller's CFL choice)
 *   stream     cudaStream_t as void* (NULL: default stream); each call waits for this stream
 *              to finish before it returns (it reads the step's status word back)
 * What it runs: S2O4 with the GKS2D flux, the DF variants (use_df = 1) of WENO5/7/9, Euler or
 * Navier-Stokes collision time (with the Prandtl fix), boundary kinds HOS_BC_FREE,
 * HOS_BC_PERIODIC, HOS_BC_REFLECT and HOS_BC_INFLOW.  Other settings (other time marching, LF,
 * use_df = 0, wedge and no-slip sides), problems with nodex or nodey above
 * HOS_STATIC_MAX_NODE and ghost above HOS_STATIC_MAX_GHOST are rejected with HOS_E_CONFIG.
 * Each call waits for its stream to finish before it returns.  The first call on a device
 * also sets up that device (looks up the array's address): make it before any stream
 * capture.  All calls share the one array and it keeps the last call's contents, so calls
 * that overlap on the GPU (other streams, other host threads) race: serialise them per
 * device.  Errors are described by hos_static_last_error(). */
#define HOS_STATIC_MAX_NODE 256
#define HOS_STATIC_MAX_GHOST 5
int hos2d_step_static(const hos_params2d* params, int precision, double* d_W, double* d_alpha_x,
                      double* d_alpha_y, double dt, void* stream);
const char* hos_static_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* HOS_GB300_H */
