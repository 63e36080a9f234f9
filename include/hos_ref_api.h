/*
 * hos_ref_api.h -- the reference's own C++ function-level API for the 1D/2D hot path
 * (XJTUZhangHong/high-order-solver), implemented by libhos_ref.so on top of the C ABI in
 * hos_gb300.h.  A driver written against the reference (the loop of PlanarShock,
 * src/2Dproblem.cpp:102-159, or SodTubeProblem, src/1Dproblem.cpp:78-148) links against
 * libhos_ref.so instead of the reference's reconstruction.cpp, flux_function.cpp,
 * time_advance.cpp, boundary_condition.cpp and the mesh/allocation parts of basic_function.cpp
 * and fluid_mesh.cpp, and runs its steps on the GPU unchanged.
 *
 * How the calls map onto the GPU (all names below are the reference's):
 *   Get_CFL (src/time_advance.cpp:75-111, 264-305) ....... first call for a Fluid array creates
 *        the device solver and uploads convar/primvar/alpha; every call fixes the step's dt on
 *        the device (hos2d_begin_step / hos1d_begin_step) and returns it.
 *   the BoundaryCondition(2d) functions (src/boundary_condition.cpp) record the boundary kind
 *        of their side; the device fills the ghost cells inside the stage.
 *   Convar_to_Primvar, Reconstruction_within_cell, Reconstruction_forg0, Calculate_flux,
 *        Update_alpha ...................................... validate the call order; their work
 *        is fused into the device stage.
 *   Update(fluids, ..., stage) (src/time_advance.cpp:113-194, 307-429) runs the fused S2O4 stage
 *        (hos2d_stage / hos1d_stage); after the last stage the new state is copied back into the
 *        Fluid array (convar, primvar, alpha_x/alpha_y or alpha) unless mirroring is off.
 *   CopyFluid_new_to_old (src/basic_function.cpp:1557-1584) copies convar to convar_old on the
 *        host while mirroring is on (the device keeps its own copy).
 * The device copy of the state is authoritative between steps: a driver that edits the Fluid
 * array between steps calls hos_ref_upload2d / hos_ref_upload1d afterwards.
 *
 * Errors follow the reference by default: a blow-up prints "the program blows up at t=...!"
 * and calls exit(0) (src/basic_function.cpp:768-772); configuration the GPU path does not
 * provide prints a message and exits likewise.  hos_ref_set_error_mode(HOS_REF_THROW) makes
 * the same conditions throw hos_ref_error instead.
 *
 * Provided: WENO5/7/9-AO with the discontinuity-feedback factor (WENO5-AO without it in 1D),
 * first-order reconstruction (First_order_normal / _tangent, the drivers' step 0), GKS2D with
 * the Euler or NS collision time (Mu / Nu, is_Prandtl_fix / Pr), GKS (1D) and LF2D; S2O4 (1D,
 * 2D) and S1O1, S1O2, RK2, RK3, RK4 (2D); free / periodic / reflective / inflow / no-slip
 * adiabatic boundaries, RT_boundary, Update_with_source (gravity source, S2O4); the output
 * writers.
 * Not provided (rejected at the first step): Van Leer reconstruction, GKS2D_smooth, LF2D's
 * viscous term, the 1D LF flux and 1D RK integrators, the 3D C++ API (the 3D path is the C ABI
 * hos3d_*).
 */
#ifndef HOS_REF_API_H
#define HOS_REF_API_H

#include <stdexcept>
#include <string>

#include "hos_gb300.h"
#include "hos_ref_types.h"

/* ---- globals the reference's drivers set (same names, types and initial values) ---- */
extern int K;                                   /* src/basic_function.cpp:3-13 */
extern double Gamma;
extern double T_inf;
extern double R_gas;
extern double Mu;
extern double Nu;
extern double c1_euler;
extern double c2_euler;
extern bool is_Prandtl_fix;
extern double Pr;
extern TAU_TYPE tau_type;
extern int gausspoint;                          /* src/fluid_mesh.cpp:3-5 */
extern double* gauss_loc;
extern double* gauss_weight;
extern Reconstruction_variable reconstruction_variable;   /* src/reconstruction.cpp:4-11, 1410-1413 */
extern WENOtype wenotype;
extern double df_thres;
extern bool is_reduce_order_warning;
extern bool is_using_df_factor;
extern bool smooth;
extern Reconstruction_within_Cell cellreconstruction;
extern Reconstruction_forG0 g0reconstruction;
extern Reconstruction_within_Cell_2D_normal cellreconstruction_2D_normal;
extern Reconstruction_within_Cell_2D_tangent cellreconstruction_2D_tangent;
extern Reconstruction_forG0_2D_normal g0reconstruction_2D_normal;
extern Reconstruction_forG0_2D_tangent g0reconstruction_2D_tangent;
extern G0_construct_type g0type;
extern GKS1d_type gks1dsolver;                  /* src/flux_function.cpp:4-5, 314-315 */
extern Flux_function flux_function;
extern GKS2d_type gks2dsolver;
extern Flux_function_2d flux_function_2d;
extern TimeMarchingCoefficient timecoe_list;    /* src/time_advance.cpp:4, 197 */
extern TimeMarchingCoefficient_2d timecoe_list_2d;

/* ---- data model: allocation and uniform mesh (src/basic_function.cpp:1262-1491,
 *      src/fluid_mesh.cpp:9-45) ---- */
void SetGuassPoint();
Flux1d** Setflux_array(Block1d block);
void SetUniformMesh(Block1d block, Fluid1d* fluids, Interface1d* interfaces, Flux1d** fluxes);
Fluid2d* Setfluid(Block2d& block);
Interface2d* Setinterface_array(Block2d block);
Flux2d_gauss** Setflux_gauss_array(Block2d block);
void SetUniformMesh(Block2d& block, Fluid2d* fluids, Interface2d* xinterfaces, Interface2d* yinterfaces,
                    Flux2d_gauss** xfluxes, Flux2d_gauss** yfluxes);
void CopyFluid_new_to_old(Fluid1d* fluids, Block1d block);
void CopyFluid_new_to_old(Fluid2d* fluids, Block2d block);
void Convar_to_Primvar(Fluid2d* fluids, Block2d block);

/* ---- time marching (src/time_advance.cpp) ---- */
void S1O1(Block1d& block);
void S1O2(Block1d& block);
void S2O4(Block1d& block);
void RK2(Block1d& block);
void RK3(Block1d& block);
void RK4(Block1d& block);
void Initial_stages(Block1d& block);
double Get_CFL(Block1d& block, Fluid1d* fluids, double tstop);
void Update(Fluid1d* fluids, Flux1d** fluxes, Block1d block, int stage);
void S1O1_2D(Block2d& block);
void S1O2_2D(Block2d& block);
void RK2_2D(Block2d& block);
void S2O4_2D(Block2d& block);
void RK4_2D(Block2d& block);
void RK3_2D(Block2d& block);
void Initial_stages(Block2d& block);
double Get_CFL(Block2d& block, Fluid2d* fluids, double tstop);
void Update(Fluid2d* fluids, Flux2d_gauss** xfluxes, Flux2d_gauss** yfluxes, Block2d block, int stage);
void Update_with_source(Fluid2d* fluids, Flux2d_gauss** xfluxes, Flux2d_gauss** yfluxes, Block2d block, int stage);

/* ---- reconstruction (src/reconstruction.cpp) ---- */
void Reconstruction_within_cell(Interface1d* interfaces, Fluid1d* fluids, Block1d block);
void Reconstruction_forg0(Interface1d* interfaces, Fluid1d* fluids, Block1d block);
void Update_alpha(Interface1d* interfaces, Fluid1d* fluids, Block1d block);
void Vanleer(Point1d& left, Point1d& right, Fluid1d* fluids, Block1d block);
void WENO5_AO(Point1d& left, Point1d& right, Fluid1d* fluids, Block1d block);
void WENO5_AO_with_DF(Point1d& left, Point1d& right, Fluid1d* fluids, Block1d block);
void WENO7_AO_with_DF(Point1d& left, Point1d& right, Fluid1d* fluids, Block1d block);
void WENO9_AO_with_DF(Point1d& left, Point1d& right, Fluid1d* fluids, Block1d block);
void Center_collision(Interface1d& interfaces, Fluid1d* fluids);

void Reconstruction_within_cell(Interface2d* xinterfaces, Interface2d* yinterfaces, Fluid2d* fluids, Block2d block);
void Reconstruction_forg0(Interface2d* xinterfaces, Interface2d* yinterfaces, Fluid2d* fluids, Block2d block);
void Update_alpha(Interface2d* xinterfaces, Interface2d* yinterfaces, Fluid2d* fluids, Block2d block);
void First_order_normal(Interface2d& left, Interface2d& right, Interface2d& down, Interface2d& up, Fluid2d* fluids,
                        Block2d block);
void WENO5_AO_normal(Interface2d& left, Interface2d& right, Interface2d& down, Interface2d& up, Fluid2d* fluids,
                     Block2d block);
void WENO5_AO_with_df_normal(Interface2d& left, Interface2d& right, Interface2d& down, Interface2d& up,
                             Fluid2d* fluids, Block2d block);
void WENO7_AO_with_df_normal(Interface2d& left, Interface2d& right, Interface2d& down, Interface2d& up,
                             Fluid2d* fluids, Block2d block);
void WENO9_AO_with_df_normal(Interface2d& left, Interface2d& right, Interface2d& down, Interface2d& up,
                             Fluid2d* fluids, Block2d block);
void First_order_tangent(Interface2d* left, Interface2d* right, Interface2d* down, Interface2d* up, Fluid2d* fluids,
                         Block2d block);
void WENO5_AO_tangent(Interface2d* left, Interface2d* right, Interface2d* down, Interface2d* up, Fluid2d* fluids,
                      Block2d block);
void WENO5_AO_with_df_tangent(Interface2d* left, Interface2d* right, Interface2d* down, Interface2d* up,
                              Fluid2d* fluids, Block2d block);
void WENO7_AO_with_df_tangent(Interface2d* left, Interface2d* right, Interface2d* down, Interface2d* up,
                              Fluid2d* fluids, Block2d block);
void WENO9_AO_with_df_tangent(Interface2d* left, Interface2d* right, Interface2d* down, Interface2d* up,
                              Fluid2d* fluids, Block2d block);
void Center_do_nothing_normal(Interface2d* xinterfaces, Interface2d* yinterfaces, Fluid2d* fluids, Block2d block);
void Center_all_collision_multi(Interface2d* xinterfaces, Interface2d* yinterfaces, Fluid2d* fluids, Block2d block);

/* ---- flux (src/flux_function.cpp) ---- */
void Calculate_flux(Flux1d** fluxes, Interface1d* interfaces, Block1d& block, int stage);
void GKS(Flux1d& flux, Interface1d& interface, double dt);
void LF(Flux1d& flux, Interface1d& interface, double dt);
void Calculate_flux(Flux2d_gauss** xfluxes, Flux2d_gauss** yfluxes, Interface2d* xinterfaces,
                    Interface2d* yinterfaces, Block2d block, int stage);
void GKS2D_smooth(Flux2d& flux, Recon2d& interface, double dt);
void GKS2D(Flux2d& flux, Recon2d& interface, double dt);
void LF2D(Flux2d& flux, Recon2d& interface, double dt);

/* ---- output writers (src/output.cpp:3-84): same file names, order and formatting ---- */
void output1d(Fluid1d* fluids, Block1d block);
void output2d(Fluid2d* fluids, Block2d block);
void output_error_form(double CFL, double dt_ratio, int mesh_set, int* mesh_number, double** error);

/* ---- boundary conditions (src/boundary_condition.cpp) ---- */
void free_boundary_left(Fluid1d* fluids, Block1d block, Fluid1d bcvalue);
void free_boundary_right(Fluid1d* fluids, Block1d block, Fluid1d bcvalue);
void reflection_boundary_left(Fluid1d* fluids, Block1d block, Fluid1d bcvalue);
void reflection_boundary_right(Fluid1d* fluids, Block1d block, Fluid1d bcvalue);
void periodic_boundary_left(Fluid1d* fluids, Block1d block, Fluid1d bcvalue);
void periodic_boundary_right(Fluid1d* fluids, Block1d block, Fluid1d bcvalue);
void free_boundary_left(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void free_boundary_right(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void free_boundary_down(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void free_boundary_up(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void periodic_boundary_left(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void periodic_boundary_right(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void periodic_boundary_down(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void periodic_boundary_up(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void inflow_boundary_left(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void inflow_boundary_right(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void inflow_boundary_up(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void reflection_boundary_up(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void reflection_boundary_down(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void reflection_boundary_right(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void reflection_boundary_left(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void noslip_adiabatic_boundary_left(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void noslip_adiabatic_boundary_right(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void noslip_adiabatic_boundary_down(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void noslip_adiabatic_boundary_up(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);
void RT_boundary(Fluid2d* fluids, Block2d block);

/* ---- controls of this library (no counterpart in the reference) ---- */
#define HOS_REF_EXIT 0    /* print and exit(0) where the reference does (default) */
#define HOS_REF_THROW 1   /* throw hos_ref_error instead                          */

class hos_ref_error : public std::runtime_error {
public:
    hos_ref_error(int code, const std::string& what) : std::runtime_error(what), code(code) {}
    int code;   /* HOS_E_* */
};

extern "C" {
/* compute precision of reconstruction and flux for solvers created afterwards (HOS_FP64 default) */
void hos_ref_set_precision(int precision);
/* 1 (default): copy the state back into the Fluid array after every step; 0: keep it on the
 * device until hos_ref_download2d / hos_ref_download1d */
void hos_ref_set_mirror(int on);
void hos_ref_set_error_mode(int mode);
/* the reference's doubleMach boundary (boundaryforDoubleMach, src/2Dproblem.cpp:1029-1093) is a
 * function of its driver, not a BoundaryCondition2d: declare it for a Fluid array before the
 * first step; the down/up boundary functions the driver calls are then ignored */
int hos_ref_set_wedge2d(const Fluid2d* fluids, double x0, double top_speed, const double* post_prim,
                        const double* pre_prim);
int hos_ref_download2d(Fluid2d* fluids, Block2d block);
int hos_ref_upload2d(Fluid2d* fluids, Block2d block);
int hos_ref_download1d(Fluid1d* fluids, Block1d block);
int hos_ref_upload1d(Fluid1d* fluids, Block1d block);
/* drop the device solver of a Fluid array (the next Get_CFL starts from the host arrays) */
void hos_ref_release(const void* fluids);
/* the device solver behind a Fluid array (NULL before its first Get_CFL) */
hos_solver2d* hos_ref_solver2d(const Fluid2d* fluids);
hos_solver1d* hos_ref_solver1d(const Fluid1d* fluids);
}

#endif /* HOS_REF_API_H */
