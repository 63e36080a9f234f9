// ref_driver.cpp -- non-interactive driver over the UNMODIFIED reference sources.
//
// TEST INFRASTRUCTURE ONLY (built into oracle/_ref/, never shipped, never linked by the
// product).  It compiles against the reference's own headers and calls the reference's own
// stage functions in exactly the order of the reference time loop
// (src/2Dproblem.cpp:128-157, PlanarShock), replacing only the interactive `cin` gate and
// the hard-wired problem setup.  Globals are set the way the reference drivers set them
// (src/2Dproblem.cpp:16-53 and :1357-1418).
#include "2Dproblem.h"
#include <cstring>
#include <vector>
#include "oracle_api.h"

namespace {
Block2d g_block;
Fluid2d* g_fluids = nullptr;
Interface2d* g_xif = nullptr;
Interface2d* g_yif = nullptr;
Flux2d_gauss** g_xfl = nullptr;
Flux2d_gauss** g_yfl = nullptr;
Fluid2d g_bcvalue[4];
int g_bc[4];

void apply_bc(int side) {
    Fluid2d* f = g_fluids;
    Block2d b = g_block;
    Fluid2d v = g_bcvalue[side];
    switch (g_bc[side]) {
    case HOS_BC_FREE:
        if (side == 0) free_boundary_left(f, b, v);
        if (side == 1) free_boundary_right(f, b, v);
        if (side == 2) free_boundary_down(f, b, v);
        if (side == 3) free_boundary_up(f, b, v);
        break;
    case HOS_BC_PERIODIC:
        if (side == 0) periodic_boundary_left(f, b, v);
        if (side == 1) periodic_boundary_right(f, b, v);
        if (side == 2) periodic_boundary_down(f, b, v);
        if (side == 3) periodic_boundary_up(f, b, v);
        break;
    case HOS_BC_REFLECT:
        if (side == 0) reflection_boundary_left(f, b, v);
        if (side == 1) reflection_boundary_right(f, b, v);
        if (side == 2) reflection_boundary_down(f, b, v);
        if (side == 3) reflection_boundary_up(f, b, v);
        break;
    case HOS_BC_INFLOW:
        if (side == 0) inflow_boundary_left(f, b, v);
        if (side == 1) inflow_boundary_right(f, b, v);
        if (side == 3) inflow_boundary_up(f, b, v);
        break;
    case HOS_BC_NOSLIP:
        if (side == 0) noslip_adiabatic_boundary_left(f, b, v);
        if (side == 1) noslip_adiabatic_boundary_right(f, b, v);
        if (side == 2) noslip_adiabatic_boundary_down(f, b, v);
        if (side == 3) noslip_adiabatic_boundary_up(f, b, v);
        break;
    }
}
}  // namespace

extern "C" {

// the WENO slots ref2d_init chose, restored by ref2d_set_first_order(0)
Reconstruction_within_Cell_2D_normal g_weno_normal = nullptr;
Reconstruction_within_Cell_2D_tangent g_weno_tangent = nullptr;

// Update_with_source in place of Update (the RT_instability loop, src/2Dproblem.cpp:752-758)
int g_source = 0;
void ref2d_set_source(int on) { g_source = on; }

// the drivers' step-0 switch (e.g. src/2Dproblem.cpp:733-745)
void ref2d_set_first_order(int on) {
    cellreconstruction_2D_normal = on ? First_order_normal : g_weno_normal;
    cellreconstruction_2D_tangent = on ? First_order_tangent : g_weno_tangent;
}

int ref2d_init(const hos2d_params* p) {
    Block2d block;
    block.uniform = true;
    block.nodex = p->nodex;
    block.nodey = p->nodey;
    block.ghost = p->ghost;
    block.CFL = p->cfl;
    K = p->K;
    Gamma = p->gamma;
    for (int s = 0; s < 4; ++s) {
        g_bc[s] = p->bc[s];
        for (int v = 0; v < 4; ++v) g_bcvalue[s].primvar[v] = p->bc_prim[s][v];
    }
    gausspoint = p->gausspoint;
    SetGuassPoint();
    reconstruction_variable = p->characteristic ? characteristic : conservative;
    wenotype = p->wenotype == 1 ? wenojs : p->wenotype == 2 ? linear : wenoz;
    is_using_df_factor = p->use_df != 0;
    if (p->order == 5) {
        cellreconstruction_2D_normal = p->use_df ? WENO5_AO_with_df_normal : WENO5_AO_normal;
        cellreconstruction_2D_tangent = p->use_df ? WENO5_AO_with_df_tangent : WENO5_AO_tangent;
    } else if (p->order == 7) {
        cellreconstruction_2D_normal = WENO7_AO_with_df_normal;
        cellreconstruction_2D_tangent = WENO7_AO_with_df_tangent;
    } else if (p->order == 9) {
        cellreconstruction_2D_normal = WENO9_AO_with_df_normal;
        cellreconstruction_2D_tangent = WENO9_AO_with_df_tangent;
    } else {
        return 2;
    }
    g_weno_normal = cellreconstruction_2D_normal;
    g_weno_tangent = cellreconstruction_2D_tangent;
    g0reconstruction_2D_normal = Center_do_nothing_normal;
    g0reconstruction_2D_tangent = Center_all_collision_multi;
    is_reduce_order_warning = false;
    gks2dsolver = gks2nd_2d;
    tau_type = p->tau_type == 1 ? NS : Euler;
    Mu = p->mu;
    Nu = p->nu;
    c1_euler = p->c1_euler;
    c2_euler = p->c2_euler;
    is_Prandtl_fix = p->prandtl_fix != 0;
    Pr = p->prandtl;
    flux_function_2d = p->flux == 1 ? LF2D : GKS2D;
    switch (p->integrator) {
        case 0: timecoe_list_2d = S2O4_2D; break;
        case 1: timecoe_list_2d = S1O1_2D; break;
        case 2: timecoe_list_2d = S1O2_2D; break;
        case 3: timecoe_list_2d = RK2_2D; break;
        case 4: timecoe_list_2d = RK3_2D; break;
        case 5: timecoe_list_2d = RK4_2D; break;
        default: return 2;
    }
    Initial_stages(block);
    block.nx = block.nodex + 2 * block.ghost;
    block.ny = block.nodey + 2 * block.ghost;
    g_fluids = Setfluid(block);
    g_xif = Setinterface_array(block);
    g_yif = Setinterface_array(block);
    g_xfl = Setflux_gauss_array(block);
    g_yfl = Setflux_gauss_array(block);
    block.left = p->left;
    block.right = p->right;
    block.down = p->down;
    block.up = p->up;
    block.dx = (block.right - block.left) / block.nodex;
    block.dy = (block.up - block.down) / block.nodey;
    block.overdx = 1 / block.dx;
    block.overdy = 1 / block.dy;
    SetUniformMesh(block, g_fluids, g_xif, g_yif, g_xfl, g_yfl);
    block.t = 0;
    block.step = 0;
    g_block = block;
    return 0;
}

void ref2d_free(void) {
    // The reference never frees its arrays; the harness process exits instead.
    g_fluids = nullptr;
}

void ref2d_set_threads(int n) { omp_set_num_threads(n); }

void ref2d_set_state(const double* convar, const double* primvar) {
    const int n = g_block.nx * g_block.ny;
    for (int c = 0; c < n; ++c)
        for (int v = 0; v < 4; ++v) {
            g_fluids[c].convar[v] = convar[4 * c + v];
            if (primvar) g_fluids[c].primvar[v] = primvar[4 * c + v];
        }
}

void ref2d_get_state(double* convar, double* primvar, double* alpha_x, double* alpha_y) {
    const int n = g_block.nx * g_block.ny;
    for (int c = 0; c < n; ++c) {
        for (int v = 0; v < 4; ++v) {
            if (convar) convar[4 * c + v] = g_fluids[c].convar[v];
            if (primvar) primvar[4 * c + v] = g_fluids[c].primvar[v];
        }
        if (alpha_x) alpha_x[c] = g_fluids[c].alpha_x;
        if (alpha_y) alpha_y[c] = g_fluids[c].alpha_y;
    }
}

double ref2d_begin_step(double tstop, double t) {
    g_block.t = t;
    CopyFluid_new_to_old(g_fluids, g_block);
    g_block.dt = Get_CFL(g_block, g_fluids, tstop);
    return g_block.dt;
}

int ref2d_stage(int stage, double dt) {
    g_block.dt = dt;
    if (g_bc[3] == HOS_BC_WEDGE_TOP) {
        // the reference's own double-Mach boundary (Mach 10 states hard-wired in it)
        boundaryforDoubleMach(g_fluids, g_block, g_bcvalue[0]);
    } else if (g_source) {
        // the RT_instability loop's own boundary (src/boundary_condition.cpp:188-242): reflecting
        // sides, fixed bottom and top states
        RT_boundary(g_fluids, g_block);
    } else {
        for (int s = 0; s < 4; ++s) apply_bc(s);
    }
    // Convar_to_Primvar exits the process on a blow-up (src/basic_function.cpp:768-772);
    // the harness checks first and reports a status instead.
    const int n = g_block.nx * g_block.ny;
    for (int c = 0; c < n; ++c) {
        double prim[4];
        Convar_to_primvar_2D(prim, g_fluids[c].convar);
        if (negative_density_or_pressure(prim)) return 1;
    }
    Convar_to_Primvar(g_fluids, g_block);
    Reconstruction_within_cell(g_xif, g_yif, g_fluids, g_block);
    Reconstruction_forg0(g_xif, g_yif, g_fluids, g_block);
    if (flux_function_2d == LF2D && tau_type == NS) {
        // LF2D's viscous term (NS_by_central_difference_prim_2D) reads each Gauss point's
        // centre state, which Center_all_collision_multi fills only when the flux is GKS2D
        // (src/reconstruction.cpp:3642-3650); the reference leaves it as allocated
        // (uninitialised).  The harness fills it with the reference's own
        // Center_all_collision_2d_multi on every face Calculate_flux evaluates.
        const Block2d b = g_block;
#pragma omp parallel for
        for (int i = b.ghost; i < b.nodex + b.ghost + 1; i++)
            for (int j = b.ghost; j < b.nodey + b.ghost; j++)
                for (int m = 0; m < gausspoint; m++) Center_all_collision_2d_multi(g_xif[i * (b.ny + 1) + j].gauss[m]);
#pragma omp parallel for
        for (int i = b.ghost; i < b.nodex + b.ghost; i++)
            for (int j = b.ghost; j < b.nodey + b.ghost + 1; j++)
                for (int m = 0; m < gausspoint; m++) Center_all_collision_2d_multi(g_yif[i * (b.ny + 1) + j].gauss[m]);
    }
    Calculate_flux(g_xfl, g_yfl, g_xif, g_yif, g_block, stage);
    if (g_source) Update_with_source(g_fluids, g_xfl, g_yfl, g_block, stage);
    else Update(g_fluids, g_xfl, g_yfl, g_block, stage);
    if (is_using_df_factor) Update_alpha(g_xif, g_yif, g_fluids, g_block);
    return 0;
}

int ref2d_step(double tstop, double t, double* dt_out) {
    double dt = ref2d_begin_step(tstop, t);
    if (dt_out) *dt_out = dt;
    for (int s = 0; s < g_block.stages; ++s) {
        int st = ref2d_stage(s, dt);
        if (st) return st;
    }
    g_block.step++;
    return 0;
}

void ref2d_get_gauss(int dir, double* out) {
    Interface2d* itf = dir == 0 ? g_xif : g_yif;
    const int nf = (g_block.nx + 1) * (g_block.ny + 1);
    for (int f = 0; f < nf; ++f)
        for (int g = 0; g < gausspoint; ++g) {
            double* o = out + (static_cast<size_t>(f) * gausspoint + g) * 36;
            Point2d* pts[3] = {&itf[f].gauss[g].left, &itf[f].gauss[g].right, &itf[f].gauss[g].center};
            for (int s = 0; s < 3; ++s)
                for (int v = 0; v < 4; ++v) {
                    o[s * 12 + v] = pts[s]->convar[v];
                    o[s * 12 + 4 + v] = pts[s]->der1x[v];
                    o[s * 12 + 8 + v] = pts[s]->der1y[v];
                }
        }
}

void ref2d_get_flux(int dir, int stage, double* out) {
    Flux2d_gauss** fl = dir == 0 ? g_xfl : g_yfl;
    const int nf = (g_block.nx + 1) * (g_block.ny + 1);
    for (int f = 0; f < nf; ++f)
        for (int g = 0; g < gausspoint; ++g) {
            double* o = out + (static_cast<size_t>(f) * gausspoint + g) * 8;
            for (int v = 0; v < 4; ++v) {
                o[v] = fl[f][stage].gauss[g].f[v];
                o[4 + v] = fl[f][stage].gauss[g].derf[v];
            }
        }
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// 1D: the loop body of SodTubeProblem / accuracy_sinwave_1d (src/1Dproblem.cpp:93-131,
// :606-640): CopyFluid_new_to_old, Get_CFL, the scheme switch after step 0, and per stage
// the two boundary calls, Reconstruction_within_cell, Reconstruction_forg0, Calculate_flux,
// Update and (when the driver uses it) Update_alpha.
// ---------------------------------------------------------------------------------------
namespace {
Block1d g_b1;
Fluid1d* g_f1 = nullptr;
Interface1d* g_i1 = nullptr;
Flux1d** g_fl1 = nullptr;
hos1d_params g_p1;
}  // namespace

extern "C" {

int ref1d_init(const hos1d_params* p) {
    g_p1 = *p;
    Block1d block;
    block.nodex = p->nodex;
    block.ghost = p->ghost;
    block.CFL = p->cfl;
    K = p->K;
    Gamma = p->gamma;
    gks1dsolver = gks2nd;
    tau_type = Euler;
    c1_euler = p->c1_euler;
    c2_euler = p->c2_euler;
    wenotype = p->wenotype == 1 ? wenojs : p->wenotype == 2 ? linear : wenoz;
    reconstruction_variable = p->characteristic ? characteristic : conservative;
    g0reconstruction = Center_collision;
    flux_function = GKS;
    timecoe_list = S2O4;
    Initial_stages(block);
    block.nx = block.nodex + 2 * block.ghost;
    block.nodex_begin = block.ghost;
    block.nodex_end = block.nodex + block.ghost - 1;
    g_f1 = new Fluid1d[block.nx];
    g_i1 = new Interface1d[block.nx + 1];
    g_fl1 = Setflux_array(block);
    block.left = p->left;
    block.right = p->right;
    block.dx = (block.right - block.left) / block.nodex;
    SetUniformMesh(block, g_f1, g_i1, g_fl1);
    block.t = 0;
    block.step = 0;
    g_b1 = block;
    return 0;
}

void ref1d_set_state(const double* convar) {
    for (int i = 0; i < g_b1.nx; ++i)
        for (int v = 0; v < 3; ++v) g_f1[i].convar[v] = convar[3 * i + v];
}

void ref1d_get_state(double* convar, double* alpha) {
    for (int i = 0; i < g_b1.nx; ++i) {
        for (int v = 0; v < 3; ++v)
            if (convar) convar[3 * i + v] = g_f1[i].convar[v];
        if (alpha) alpha[i] = g_f1[i].alpha;
    }
}

int ref1d_step(double tstop, double t, int step, double* dt_out) {
    g_b1.t = t;
    g_b1.step = step;
    CopyFluid_new_to_old(g_f1, g_b1);
    g_b1.dt = Get_CFL(g_b1, g_f1, tstop);
    if (dt_out) *dt_out = g_b1.dt;
    const bool df = g_p1.df_mode == 1 || (g_p1.df_mode == 2 && step > 0);
    using Recon1 = Reconstruction_within_Cell;
    if (g_p1.order == 5) cellreconstruction = df ? static_cast<Recon1>(WENO5_AO_with_DF) : static_cast<Recon1>(WENO5_AO);
    else if (g_p1.order == 7) cellreconstruction = static_cast<Recon1>(WENO7_AO_with_DF);
    else cellreconstruction = static_cast<Recon1>(WENO9_AO_with_DF);
    Fluid1d bcv;
    for (int i = 0; i < g_b1.stages; ++i) {
        for (int side = 0; side < 2; ++side) {
            const int kind = g_p1.bc[side];
            if (kind == HOS_BC_FREE) {
                if (side) free_boundary_right(g_f1, g_b1, bcv); else free_boundary_left(g_f1, g_b1, bcv);
            } else if (kind == HOS_BC_PERIODIC) {
                if (side) periodic_boundary_right(g_f1, g_b1, bcv); else periodic_boundary_left(g_f1, g_b1, bcv);
            } else {
                if (side) reflection_boundary_right(g_f1, g_b1, bcv); else reflection_boundary_left(g_f1, g_b1, bcv);
            }
        }
        Reconstruction_within_cell(g_i1, g_f1, g_b1);
        Reconstruction_forg0(g_i1, g_f1, g_b1);
        Calculate_flux(g_fl1, g_i1, g_b1, i);
        Update(g_f1, g_fl1, g_b1, i);
        if (g_p1.update_alpha) Update_alpha(g_i1, g_f1, g_b1);
    }
    return 0;
}

}  // extern "C"
