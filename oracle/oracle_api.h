/*
 * oracle_api.h -- C interface of the CPU oracle for the 2D GKS / WENO-AO / S2O4 step.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the checker for the CUDA path; nothing in the
 * product (the hos_gb300 package and its CUDA library) includes, links or calls it.
 * Two libraries implement this interface:
 *   - liboracle.so    : the repository's own FP64 restatement (hos_oracle2d.cpp), which
 *                       builds on any host and travels with the repository;
 *   - _ref/libhosref.so : the unmodified reference sources compiled from where they lie plus
 *                       a non-interactive driver (ref_driver.cpp); it only builds where the
 *                       reference checkout exists and pins the restatement.
 * Both export the same symbols with prefixes "oracle2d_" and "ref2d_".
 *
 * State layout is the reference's own: cell (i, j) at i*ny + j (y fastest) over the full
 * block including ghost cells, 4 doubles per cell (rho, rho*u, rho*v, rho*E) -- the AoS
 * order of Fluid2d::convar (include/fluid_mesh.h:125-160 in the reference).
 */
#ifndef HOS_ORACLE_API_H
#define HOS_ORACLE_API_H

#ifdef __cplusplus
extern "C" {
#endif

/* Boundary kinds, one per side (left, right, down, up). */
enum { HOS_BC_FREE = 0, HOS_BC_PERIODIC = 1, HOS_BC_REFLECT = 2, HOS_BC_INFLOW = 3,
       HOS_BC_WEDGE_BOTTOM = 4, HOS_BC_WEDGE_TOP = 5, HOS_BC_NOSLIP = 6 };

typedef struct hos2d_params {
    int nodex, nodey;     /* interior cells                                  */
    int ghost;            /* ghost layers per side (reference drivers use 5) */
    int order;            /* WENO-AO order: 5, 7 or 9                        */
    int gausspoint;       /* Gauss points per face: 2 (5th), 3 (7th), 4 (9th)*/
    int characteristic;   /* 1: characteristic variables, 0: conservative    */
    int use_df;           /* 1: discontinuity-feedback variants; 0: non-DF WENO5-AO (order 5) */
    int K;                /* internal degrees of freedom (2D: K = 3 for gamma 1.4) */
    double gamma;
    double c1_euler, c2_euler;  /* numerical collision time coefficients     */
    double cfl;
    double left, right, down, up;
    int bc[4];            /* left, right, down, up                           */
    double bc_prim[4][4]; /* inflow primitive state per side (rho,u,v,p)     */
    /* wedge (double-Mach) boundaries, kinds 4 (bottom) and 5 (top) */
    double wedge_x0, wedge_top_speed, wedge_post[4], wedge_pre[4];
    /* time marching: 0 S2O4, 1 S1O1, 2 S1O2, 3 RK2, 4 RK3, 5 RK4; flux: 0 GKS2D, 1 LF2D */
    int integrator, flux;
    /* collision time: 0 Euler, 1 Navier-Stokes with Mu / Nu (Get_Tau_NS, Get_Tau); Prandtl
     * fix of the heat flux (is_Prandtl_fix, Pr).  No-slip walls (HOS_BC_NOSLIP) take their
     * wall velocity from bc_prim[side][1..2]. */
    int tau_type;
    double mu, nu;
    int prandtl_fix;
    double prandtl;
    /* weights of the non-DF WENO5-AO scheme (use_df = 0; the reference's wenotype):
     * 0 Z-type (wenoz), 1 Jiang-Shu (wenojs), 2 linear */
    int wenotype;
} hos2d_params;

/* ---- restatement (liboracle.so) ---- */
int    oracle2d_init(const hos2d_params* p);
void   oracle2d_free(void);
/* learned-gate features [ncell][2][16] and label distances [ncell][2] of a state (test oracle) */
void   oracle2d_gate_cells(const double* convar, const double* alpha_x, const double* alpha_y, double* feat, double* dist);
void   oracle2d_set_threads(int n);
/* 1: First_order_normal / First_order_tangent in the reconstruction slots (the drivers' step 0
 * when is_using_df_factor is set); 0: the WENO-AO scheme of the configured order */
void   oracle2d_set_first_order(int on);
/* 1: the stage update is Update_with_source (gravity source, the RT_instability driver) */
void   oracle2d_set_source(int on);
void   oracle2d_set_state(const double* convar, const double* primvar);
void   oracle2d_get_state(double* convar, double* primvar, double* alpha_x, double* alpha_y);
double oracle2d_begin_step(double tstop, double t);     /* CopyFluid_new_to_old + Get_CFL */
int    oracle2d_stage(int stage, double dt);            /* one S2O4 stage; status 0 ok   */
int    oracle2d_step(double tstop, double t, double* dt_out);
/* Gauss-point states of the last stage: per face, per Gauss point, 36 doubles
 * (left, right, centre) x (convar, der1x, der1y) x 4; faces (nx+1)*(ny+1), dir 0 = x. */
void   oracle2d_get_gauss(int dir, double* out);
/* Per-face, per-Gauss-point time-integrated flux f[4], derf[4] of stage s. */
void   oracle2d_get_flux(int dir, int stage, double* out);

/* ---- compiled reference (_ref/libhosref.so) ---- */
int    ref2d_init(const hos2d_params* p);
void   ref2d_free(void);
void   ref2d_set_threads(int n);
void   ref2d_set_first_order(int on);
void   ref2d_set_source(int on);
void   ref2d_set_state(const double* convar, const double* primvar);
void   ref2d_get_state(double* convar, double* primvar, double* alpha_x, double* alpha_y);
double ref2d_begin_step(double tstop, double t);
int    ref2d_stage(int stage, double dt);
int    ref2d_step(double tstop, double t, double* dt_out);
void   ref2d_get_gauss(int dir, double* out);
void   ref2d_get_flux(int dir, int stage, double* out);

/* ---- 1D (SodTubeProblem / accuracy_sinwave_1d, src/1Dproblem.cpp) ----
 * State: cell i at index i over the full line including ghosts, 3 doubles per cell. */
typedef struct hos1d_params {
    int nodex, ghost;
    int order;            /* 5, 7, 9 (DF variants); 5 also has the non-DF variant      */
    int characteristic;   /* 1: characteristic variables, 0: conservative              */
    int df_mode;          /* 0: non-DF WENO5-AO every step; 1: DF variant every step;
                             2: non-DF at step 0, DF from step 1 (the Sod driver)        */
    int update_alpha;     /* 1: Update_alpha after every stage (Sod); 0: never (accuracy) */
    int K;
    double gamma;
    double c1_euler, c2_euler;
    double cfl;
    double left, right;
    int bc[2];            /* left, right: HOS_BC_FREE / PERIODIC / REFLECT              */
    int wenotype;         /* non-DF steps: 0 Z-type, 1 Jiang-Shu, 2 linear weights      */
} hos1d_params;

int    oracle1d_init(const hos1d_params* p);
void   oracle1d_set_state(const double* convar);
void   oracle1d_get_state(double* convar, double* alpha);
int    oracle1d_step(double tstop, double t, int step, double* dt_out);

int    ref1d_init(const hos1d_params* p);
void   ref1d_set_state(const double* convar);
void   ref1d_get_state(double* convar, double* alpha);
int    ref1d_step(double tstop, double t, int step, double* dt_out);

/* ---- 3D (CubicTube's loop, src/3Dproblem.cpp:125-157; non-DF WENO5-AO, 2x2 Gauss
 * points per face, GKS3D, S2O4).  State: cell (i, j, k) at (i*ny + j)*nz + k over the full
 * block including ghosts, 5 doubles per cell (rho, rho u, rho v, rho w, rho E). */
typedef struct hos3d_params {
    int nodex, nodey, nodez, ghost;   /* ghost >= 3                                       */
    int characteristic;               /* 1: characteristic variables, 0: conservative     */
    int K;                            /* internal degrees of freedom (K = 2 for gamma 1.4) */
    double gamma;
    double c1_euler, c2_euler;        /* numerical collision time coefficients           */
    double cfl;
    int tau_type;                     /* 0: Euler, 1: Navier-Stokes with viscosity mu     */
    double mu;
    double left, right, down, up, back, front;
    int bc[6];                        /* left, right, down, up, back, front: FREE / PERIODIC / REFLECT */
    int prandtl_fix;                  /* 1: Prandtl-number correction of the heat flux      */
    double prandtl;                   /* Pr */
    int gks3d_pressure_slot;          /* GPU switch of the same layout; the restatement takes
                                         oracle3d_set_reference_conventions instead          */
} hos3d_params;

int    oracle3d_init(const hos3d_params* p);
void   oracle3d_free(void);
void   oracle3d_set_state(const double* convar, const double* primvar);  /* primvar may be NULL */
void   oracle3d_get_state(double* convar, double* primvar);
double oracle3d_begin_step(double tstop, double t);
int    oracle3d_stage(int stage, double dt);
int    oracle3d_step(double tstop, double t, double* dt_out);
/* 1: keep the collision time of dt at the dt/2 level (the 1D GKS convention), for comparing
 * one-dimensional 3D data with the 1D restatement; 0 (default): recompute it (GKS3D) */
void   oracle3d_set_half_tau_of_dt(int on);
/* 1: the reference's own 3D conventions (pressure in GKS3D's lambda slots, order-reduction flags
 * of lines and Gauss points that stay set once set), for comparing with the reference's 3D
 * functions run by ref_driver3d.cpp; 0 (default): lambda, each reconstruction decides afresh */
void   oracle3d_set_reference_conventions(int on);
/* number of line / Gauss-point reconstructions whose order-reduction flag is set (reference
 * conventions only) */
long long oracle3d_reduced_count(void);

/* ---- compiled reference, 3D (_ref/libhosref.so, ref_driver3d.cpp): free sides only ---- */
int    ref3d_init(const hos3d_params* p);
void   ref3d_set_threads(int n);
void   ref3d_set_state(const double* convar, const double* primvar);
void   ref3d_get_state(double* convar, double* primvar);
double ref3d_begin_step(double tstop, double t);
int    ref3d_stage(int stage, double dt);
int    ref3d_step(double tstop, double t, double* dt_out);
long long ref3d_reduced_count(void);
/* per interior face of direction dir, stage fluxes summed over the 4 Gauss points with
 * weight 1/4, in the face frame: [face][stage][f 5, derf 5]; faces ordered (normal, t1, t2)
 * with x faces (i, j, k), y faces (j, nx-1-i, k), z faces (k, j, nx-1-i) over interior cells */
void   oracle3d_get_flux(int dir, double* out);

#ifdef __cplusplus
}
#endif
#endif
