// hos_ref_path.cpp -- the per-step half of the reference's function-level API (1D and 2D):
// Get_CFL, the boundary functions, Convar_to_Primvar, Reconstruction_within_cell,
// Reconstruction_forg0, Calculate_flux, Update, Update_alpha and the function-pointer slots
// the drivers assign, implemented over the C ABI of libhos_gb300.so.  One device solver
// (hos_solver2d / hos_solver1d) stands behind each Fluid array a driver steps.
//
// The stage's work is fused on the device, so only Get_CFL (fixes dt) and Update (runs the
// stage) launch anything; the other per-stage calls record boundary kinds or check the call
// order.  After the last stage of a step the state is copied back into the Fluid array.
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "hos_ref_api.h"

// ---- function-pointer slots and switches of the replaced files, with the reference's initial
// values (src/reconstruction.cpp:4-11, 1410-1413, 3690; src/flux_function.cpp:4-5, 314-315;
// src/time_advance.cpp:4, 197) ----
Reconstruction_variable reconstruction_variable = conservative;
WENOtype wenotype = wenojs;
double df_thres = 3.0;
bool is_reduce_order_warning = false;
bool is_using_df_factor = false;
bool smooth = false;
Reconstruction_within_Cell cellreconstruction = Vanleer;
Reconstruction_forG0 g0reconstruction = Center_collision;
Reconstruction_within_Cell_2D_normal cellreconstruction_2D_normal = WENO5_AO_normal;
Reconstruction_within_Cell_2D_tangent cellreconstruction_2D_tangent = WENO5_AO_tangent;
Reconstruction_forG0_2D_normal g0reconstruction_2D_normal = Center_do_nothing_normal;
Reconstruction_forG0_2D_tangent g0reconstruction_2D_tangent = Center_all_collision_multi;
G0_construct_type g0type = all_collisionn;
GKS1d_type gks1dsolver = nothing;
Flux_function flux_function = LF;
GKS2d_type gks2dsolver = kfvs1st_2d;
Flux_function_2d flux_function_2d = GKS2D;
TimeMarchingCoefficient timecoe_list = RK2;
TimeMarchingCoefficient_2d timecoe_list_2d = S1O1_2D;

namespace {

int g_precision = HOS_FP64;
bool g_mirror = true;
int g_mode = HOS_REF_EXIT;

// The reference prints and exits (src/basic_function.cpp:768-772, src/time_advance.cpp:310-314);
// in HOS_REF_THROW mode the same condition throws.
void stop(int code, const std::string& msg) {
    if (g_mode == HOS_REF_THROW) throw hos_ref_error(code, msg);
    std::cout << msg << std::endl;
    std::exit(0);
}

void blow_up(double t) {
    std::ostringstream o;
    o << "the program blows up at t=" << t << "!";
    stop(HOS_E_BLOWUP, o.str());
}

void check2(int st, const char* what) {
    if (st != HOS_OK) stop(st, std::string(what) + ": " + hos_last_error());
}

void check1(int st, const char* what) {
    if (st != HOS_OK) stop(st, std::string(what) + ": " + hos1d_last_error());
}

void not_fused(const char* name) {
    stop(HOS_E_CONFIG, std::string(name) +
                           " is evaluated inside the fused GPU stage; assign it to its slot and call "
                           "Reconstruction_within_cell / Calculate_flux / Update");
}

struct Side {
    int kind = -1;          // HOS_BC_*, -1 not recorded, -2 not provided on the GPU path
    double prim[4] = {0, 0, 0, 0};
};

bool same(const Side& a, const Side& b) {
    if (a.kind != b.kind) return false;
    if (a.kind != HOS_BC_INFLOW && a.kind != HOS_BC_NOSLIP) return true;
    for (int v = 0; v < 4; ++v)
        if (a.prim[v] != b.prim[v]) return false;
    return true;
}

// ======================================= 2D =======================================

struct Ctx2 {
    hos_solver2d* h = nullptr;
    int nx = 0, ny = 0, order = 0;
    int use_df = 1;         // the solver's scheme: DF variants (1) or the non-DF WENO5-AO (0)
    double cfl = 0, tstop = 0;
    Side cur[4], pend[4];
    unsigned pend_mask = 0;
    int next = -1;          // stage Update expects next; -1 between steps
    bool stepped = false;   // a stage has run on this solver
    bool wedge = false;
    double wx0 = 0, wspeed = 0, wpost[4] = {0, 0, 0, 0}, wpre[4] = {0, 0, 0, 0};
    std::vector<double> con, prim, ax, ay;
    std::vector<double> prim_last;   // primitives at the start of the last stage
};
std::map<const void*, Ctx2> g_ctx2;

int order_of(Reconstruction_within_Cell_2D_normal f) {
    if (f == WENO5_AO_normal || f == WENO5_AO_with_df_normal) return 5;
    if (f == WENO7_AO_with_df_normal) return 7;
    if (f == WENO9_AO_with_df_normal) return 9;
    return 0;
}

int tangent_order_of(Reconstruction_within_Cell_2D_tangent f) {
    if (f == WENO5_AO_tangent || f == WENO5_AO_with_df_tangent) return 5;
    if (f == WENO7_AO_with_df_tangent) return 7;
    if (f == WENO9_AO_with_df_tangent) return 9;
    return 0;
}

// the problem parameters the globals and the Block2d describe (src/2Dproblem.cpp:7-81).
// First_order_normal / _tangent (the drivers' step 0 when is_using_df_factor is set,
// src/2Dproblem.cpp:733-745) run on the solver of the order whose Gauss points gausspoint
// names, which the drivers then pair with their WENO-AO-DF scheme.  Without
// is_using_df_factor the drivers keep their first slots, WENO5_AO_normal / WENO5_AO_tangent
// (the non-DF WENO5-AO with the wenotype weights), and never call Update_alpha
// (src/2Dproblem.cpp:37-38, 132-136, 154-157): the solver runs that scheme (use_df = 0).
hos_params2d params2(const Block2d& b, int* order_out, int* first_order_out = nullptr) {
    const bool fo = cellreconstruction_2D_normal == First_order_normal;
    int order;
    if (fo) {
        if (cellreconstruction_2D_tangent != First_order_tangent)
            stop(HOS_E_CONFIG, "First_order_normal goes with First_order_tangent");
        order = gausspoint == 2 ? 5 : gausspoint == 3 ? 7 : gausspoint == 4 ? 9 : 0;
        if (!order) stop(HOS_E_CONFIG, "first-order reconstruction runs with gausspoint 2, 3 or 4");
    } else {
        order = order_of(cellreconstruction_2D_normal);
        if (!order) stop(HOS_E_CONFIG, "the GPU path provides WENO5/7/9-AO and first-order reconstruction (cellreconstruction_2D_normal)");
        if (tangent_order_of(cellreconstruction_2D_tangent) != order)
            stop(HOS_E_CONFIG, "cellreconstruction_2D_tangent must be the WENO-AO variant of the normal reconstruction's order");
    }
    if (first_order_out) *first_order_out = fo ? 1 : 0;
    if (!is_using_df_factor) {
        // the reference leaves the DF indicators at zero then; the GPU path runs the slots that
        // do not read them
        if (fo || cellreconstruction_2D_normal != WENO5_AO_normal || cellreconstruction_2D_tangent != WENO5_AO_tangent)
            stop(HOS_E_CONFIG, "with is_using_df_factor = false the GPU path runs WENO5_AO_normal / WENO5_AO_tangent "
                               "(the DF variants and first order update the DF indicators: set is_using_df_factor = true)");
        if (gausspoint != 2)
            stop(HOS_E_CONFIG, "WENO5_AO_tangent writes its Gauss points only with gausspoint = 2");
    }
    if (g0reconstruction_2D_normal != Center_do_nothing_normal || g0reconstruction_2D_tangent != Center_all_collision_multi)
        stop(HOS_E_CONFIG, "the GPU path builds the GKS centre state by Center_all_collision_multi");
    if (flux_function_2d != GKS2D && flux_function_2d != LF2D)
        stop(HOS_E_CONFIG, "the GPU path provides the GKS2D and LF2D fluxes");
    if (tau_type != Euler && tau_type != NS) stop(HOS_E_CONFIG, "the GPU path provides the Euler and NS collision times");
    if (tau_type == NS && flux_function_2d == LF2D && !(Pr > 0))
        stop(HOS_E_CONFIG, "LF2D's viscous term divides by Pr: set Pr > 0");
    int integrator = -1, stages = 0;
    const TimeMarchingCoefficient_2d methods[6] = {S2O4_2D, S1O1_2D, S1O2_2D, RK2_2D, RK3_2D, RK4_2D};
    const int method_stages[6] = {2, 1, 1, 2, 3, 4};
    for (int k = 0; k < 6; ++k)
        if (timecoe_list_2d == methods[k]) {
            integrator = k;
            stages = method_stages[k];
        }
    if (integrator < 0) stop(HOS_E_CONFIG, "the GPU path provides S2O4_2D, S1O1_2D, S1O2_2D and RK2/3/4_2D time marching");
    if (b.stages != stages)
        stop(HOS_E_CONFIG, "Block2d::stages does not match timecoe_list_2d: call Initial_stages(block) after setting it");
    hos_params2d p{};
    p.integrator = integrator;
    p.flux = flux_function_2d == LF2D ? HOS_FLUX_LF : HOS_FLUX_GKS;
    p.nodex = b.nodex;
    p.nodey = b.nodey;
    p.ghost = b.ghost;
    p.order = order;
    p.gausspoint = gausspoint;
    p.characteristic = reconstruction_variable == characteristic ? 1 : 0;
    p.use_df = is_using_df_factor ? 1 : 0;
    p.wenotype = wenotype == wenojs ? HOS_WENO_JS : wenotype == linear ? HOS_WENO_LINEAR : HOS_WENO_Z;
    p.K = K;
    p.gamma = Gamma;
    p.c1_euler = c1_euler;
    p.c2_euler = c2_euler;
    p.cfl = b.CFL;
    p.tau_type = tau_type == NS ? HOS_TAU_NS : HOS_TAU_EULER;
    p.mu = Mu;
    p.nu = Nu;
    p.prandtl_fix = is_Prandtl_fix ? 1 : 0;
    p.prandtl = Pr;
    p.left = b.left;
    p.right = b.right;
    p.down = b.down;
    p.up = b.up;
    for (int s = 0; s < 4; ++s) p.bc[s] = HOS_BC_FREE;
    *order_out = order;
    return p;
}

void gather2(Ctx2& c, const Fluid2d* f) {
    const size_t n = (size_t)c.nx * c.ny;
    c.con.resize(4 * n);
    c.prim.resize(4 * n);
    c.ax.resize(n);
    c.ay.resize(n);
    for (size_t k = 0; k < n; ++k) {
        for (int v = 0; v < 4; ++v) {
            c.con[4 * k + v] = f[k].convar[v];
            c.prim[4 * k + v] = f[k].primvar[v];
        }
        c.ax[k] = f[k].alpha_x;
        c.ay[k] = f[k].alpha_y;
    }
}

void upload2(Ctx2& c, const Fluid2d* f, double t) {
    gather2(c, f);
    int st = hos2d_set_state(c.h, c.con.data(), c.prim.data());
    if (st == HOS_E_BLOWUP) blow_up(t);
    check2(st, "set_state");
    check2(hos2d_set_alpha(c.h, c.ax.data(), c.ay.data()), "set_alpha");
    check2(hos2d_set_time(c.h, t), "set_time");
}

void download2(Ctx2& c, Fluid2d* f) {
    const size_t n = (size_t)c.nx * c.ny;
    c.con.resize(4 * n);
    c.prim.resize(4 * n);
    c.ax.resize(n);
    c.ay.resize(n);
    // primvar as the reference leaves it: converted at the start of the last stage
    const bool lagged = c.prim_last.size() == 4 * n;
    check2(hos2d_get_state(c.h, c.con.data(), lagged ? nullptr : c.prim.data(), c.ax.data(), c.ay.data()),
           "get_state");
    const double* pv = lagged ? c.prim_last.data() : c.prim.data();
    for (size_t k = 0; k < n; ++k) {
        for (int v = 0; v < 4; ++v) {
            f[k].convar[v] = c.con[4 * k + v];
            f[k].primvar[v] = pv[4 * k + v];
        }
        f[k].alpha_x = c.ax[k];
        f[k].alpha_y = c.ay[k];
    }
}

void create2(Ctx2& c, const Block2d& b, const Fluid2d* f) {
    int order = 0;
    hos_params2d p = params2(b, &order);
    if (c.wedge) {
        p.bc[0] = HOS_BC_INFLOW;
        for (int v = 0; v < 4; ++v) p.bc_prim[0][v] = c.wpost[v];
        p.bc[2] = HOS_BC_WEDGE_BOTTOM;
        p.bc[3] = HOS_BC_WEDGE_TOP;
        p.wedge_x0 = c.wx0;
        p.wedge_top_speed = c.wspeed;
        for (int v = 0; v < 4; ++v) {
            p.wedge_post[v] = c.wpost[v];
            p.wedge_pre[v] = c.wpre[v];
        }
    }
    check2(hos2d_create(&p, g_precision, &c.h), "hos2d_create");
    for (int s = 0; s < 4; ++s) {
        c.cur[s].kind = p.bc[s];
        for (int v = 0; v < 4; ++v) c.cur[s].prim[v] = p.bc_prim[s][v];
    }
    c.nx = b.nx;
    c.ny = b.ny;
    c.order = order;
    c.use_df = p.use_df;
    c.cfl = b.CFL;
    c.stepped = false;
    upload2(c, f, b.t);
}

Ctx2& ctx2(const Fluid2d* f) { return g_ctx2[f]; }

// the solver exists (Update_alpha follows the last Update of a step, after it completed)
void known2(const Fluid2d* f, const char* who) {
    auto it = g_ctx2.find(f);
    if (it == g_ctx2.end() || !it->second.h)
        stop(HOS_E_CONFIG, std::string(who) + " called before the first step: Get_CFL starts each step");
}

Ctx2& live2(const Fluid2d* f, const char* who) {
    auto it = g_ctx2.find(f);
    if (it == g_ctx2.end() || !it->second.h || it->second.next < 0)
        stop(HOS_E_CONFIG, std::string(who) + " called outside a time step: Get_CFL starts each step");
    return it->second;
}

void record2(const Fluid2d* f, int side, int kind, const Fluid2d* bcvalue) {
    Ctx2& c = ctx2(f);
    c.pend[side].kind = kind;
    if ((kind == HOS_BC_INFLOW || kind == HOS_BC_NOSLIP) && bcvalue)
        for (int v = 0; v < 4; ++v) c.pend[side].prim[v] = bcvalue->primvar[v];
    c.pend_mask |= 1u << side;
}

// push the boundary kinds recorded in this stage to the device solver when they changed
void apply_boundaries2(Ctx2& c) {
    const unsigned need = c.wedge ? 0x3u : 0xFu;
    if ((c.pend_mask & need) != need)
        stop(HOS_E_CONFIG, "call the boundary function of every side before Update in each stage");
    Side want[4];
    for (int s = 0; s < 4; ++s) want[s] = c.pend[s];
    if (c.wedge) {
        want[2].kind = HOS_BC_WEDGE_BOTTOM;
        want[3].kind = HOS_BC_WEDGE_TOP;
    }
    for (int s = 0; s < 4; ++s)
        if (want[s].kind == -2)
            stop(HOS_E_CONFIG, "the GPU path provides free, periodic, reflective, inflow and no-slip adiabatic boundaries");
    bool changed = false;
    for (int s = 0; s < 4; ++s) changed |= !same(want[s], c.cur[s]);
    if (changed) {
        int kinds[4];
        double prims[16];
        for (int s = 0; s < 4; ++s) {
            kinds[s] = want[s].kind;
            for (int v = 0; v < 4; ++v) prims[4 * s + v] = want[s].prim[v];
        }
        check2(hos2d_set_boundary(c.h, kinds, prims), "boundary");
        for (int s = 0; s < 4; ++s) c.cur[s] = want[s];
    }
    c.pend_mask = 0;
}

// ======================================= 1D =======================================

struct Ctx1 {
    hos_solver1d* h = nullptr;
    int nx = 0, order = 0, df_mode = 0;
    double cfl = 0;
    long steps = 0;        // steps taken by this solver
    Side cur[2], pend[2];
    unsigned pend_mask = 0;
    int next = -1;
    std::vector<double> con, alpha;
};
std::map<const void*, Ctx1> g_ctx1;

int order1(Reconstruction_within_Cell f, bool* df) {
    *df = f != WENO5_AO;
    if (f == WENO5_AO || f == WENO5_AO_with_DF) return 5;
    if (f == WENO7_AO_with_DF) return 7;
    if (f == WENO9_AO_with_DF) return 9;
    return 0;
}

void upload1(Ctx1& c, const Fluid1d* f, double t) {
    c.con.resize(3 * (size_t)c.nx);
    c.alpha.resize(c.nx);
    for (int i = 0; i < c.nx; ++i) {
        for (int v = 0; v < 3; ++v) c.con[3 * i + v] = f[i].convar[v];
        c.alpha[i] = f[i].alpha;
    }
    int st = hos1d_set_state(c.h, c.con.data());
    if (st == HOS_E_BLOWUP) blow_up(t);
    check1(st, "set_state");
    check1(hos1d_set_alpha(c.h, c.alpha.data()), "set_alpha");
    check1(hos1d_set_time(c.h, t), "set_time");
}

void download1(Ctx1& c, Fluid1d* f) {
    c.con.resize(3 * (size_t)c.nx);
    c.alpha.resize(c.nx);
    check1(hos1d_get_state(c.h, c.con.data(), c.alpha.data()), "get_state");
    for (int i = 0; i < c.nx; ++i) {
        for (int v = 0; v < 3; ++v) f[i].convar[v] = c.con[3 * i + v];
        f[i].alpha = c.alpha[i];
    }
}

void create1(Ctx1& c, const Block1d& b, const Fluid1d* f) {
    bool df = false;
    const int order = order1(cellreconstruction, &df);
    if (!order) stop(HOS_E_CONFIG, "the GPU path provides WENO5-AO and WENO5/7/9-AO-DF reconstruction (cellreconstruction)");
    if (g0reconstruction != Center_collision) stop(HOS_E_CONFIG, "the GPU path builds the GKS centre state by Center_collision");
    if (flux_function != GKS) stop(HOS_E_CONFIG, "the GPU path provides the GKS flux");
    if (tau_type != Euler) stop(HOS_E_CONFIG, "the 1D GPU path provides the Euler collision time (tau_type = Euler)");
    if (timecoe_list != S2O4) stop(HOS_E_CONFIG, "the GPU path provides S2O4 time marching");
    if (b.stages != 2) stop(HOS_E_CONFIG, "S2O4 has two stages: call Initial_stages(block) after setting timecoe_list");
    hos_params1d p{};
    p.nodex = b.nodex;
    p.ghost = b.ghost;
    p.order = order;
    p.characteristic = reconstruction_variable == characteristic ? 1 : 0;
    // the Sod driver starts with WENO5_AO and switches to WENO5_AO_with_DF after step 0
    // (src/1Dproblem.cpp:103-106)
    p.df_mode = df ? 1 : (is_using_df_factor && b.step == 0 ? 2 : 0);
    p.update_alpha = is_using_df_factor ? 1 : 0;
    p.wenotype = wenotype == wenojs ? HOS_WENO_JS : wenotype == linear ? HOS_WENO_LINEAR : HOS_WENO_Z;
    p.K = K;
    p.gamma = Gamma;
    p.c1_euler = c1_euler;
    p.c2_euler = c2_euler;
    p.cfl = b.CFL;
    p.left = b.left;
    p.right = b.right;
    p.bc[0] = p.bc[1] = HOS_BC_FREE;
    check1(hos1d_create(&p, g_precision, &c.h), "hos1d_create");
    c.cur[0].kind = c.cur[1].kind = HOS_BC_FREE;
    c.nx = b.nx;
    c.order = order;
    c.df_mode = p.df_mode;
    c.cfl = b.CFL;
    c.steps = 0;
    upload1(c, f, b.t);
}

void known1(const Fluid1d* f, const char* who) {
    auto it = g_ctx1.find(f);
    if (it == g_ctx1.end() || !it->second.h)
        stop(HOS_E_CONFIG, std::string(who) + " called before the first step: Get_CFL starts each step");
}

Ctx1& live1(const Fluid1d* f, const char* who) {
    auto it = g_ctx1.find(f);
    if (it == g_ctx1.end() || !it->second.h || it->second.next < 0)
        stop(HOS_E_CONFIG, std::string(who) + " called outside a time step: Get_CFL starts each step");
    return it->second;
}

void record1(const Fluid1d* f, int side, int kind) {
    Ctx1& c = g_ctx1[f];
    c.pend[side].kind = kind;
    c.pend_mask |= 1u << side;
}

}  // namespace

// ======================================= 2D API =======================================

double Get_CFL(Block2d& block, Fluid2d* fluids, double tstop) {
    Ctx2& c = ctx2(fluids);
    if (c.next >= 0) stop(HOS_E_CONFIG, "Get_CFL called inside a time step");
    if (!c.h) create2(c, block, fluids);
    else if (block.nx != c.nx || block.ny != c.ny || block.CFL != c.cfl)
        stop(HOS_E_CONFIG, "the Block2d changed under a running solver: call hos_ref_release first");
    c.tstop = tstop;
    check2(hos2d_begin_step(c.h, tstop), "Get_CFL");
    double t = 0, dt = 0;
    const int st = hos2d_sync(c.h, &t, &dt);
    if (st == HOS_E_BLOWUP) blow_up(block.t);
    check2(st, "Get_CFL");
    c.next = 0;
    return dt;
}

void CopyFluid_new_to_old(Fluid2d* fluids, Block2d block) {
    if (!g_mirror) return;  // the device keeps the step's starting state itself
    for (int i = block.ghost; i < block.ghost + block.nodex; ++i)
        for (int j = block.ghost; j < block.ghost + block.nodey; ++j) {
            Fluid2d& cell = fluids[(size_t)i * block.ny + j];
            for (int v = 0; v < 4; ++v) cell.convar_old[v] = cell.convar[v];
        }
}

// fused: the device converts the state at the start of each stage
void Convar_to_Primvar(Fluid2d*, Block2d) {}

void Reconstruction_within_cell(Interface2d*, Interface2d*, Fluid2d* fluids, Block2d) {
    live2(fluids, "Reconstruction_within_cell");
}

void Reconstruction_forg0(Interface2d*, Interface2d*, Fluid2d* fluids, Block2d) {
    live2(fluids, "Reconstruction_forg0");
}

void Calculate_flux(Flux2d_gauss**, Flux2d_gauss**, Interface2d*, Interface2d*, Block2d block, int stage) {
    if (stage < 0 || stage >= block.stages)
        stop(HOS_E_CONFIG, "wrong middle stage,pls check the time marching setting");
}

namespace {
void update2(Fluid2d* fluids, Block2d block, int stage, bool source);
}

void Update(Fluid2d* fluids, Flux2d_gauss**, Flux2d_gauss**, Block2d block, int stage) {
    update2(fluids, block, stage, false);
}

// the RT_instability loop's update (src/time_advance.cpp:534-704): gravity source, S2O4 stage 0
void Update_with_source(Fluid2d* fluids, Flux2d_gauss**, Flux2d_gauss**, Block2d block, int stage) {
    update2(fluids, block, stage, true);
}

// RT_boundary (src/boundary_condition.cpp:188-242): reflecting left / right, the fixed bottom
// (rho, u, v, p) = (2, 0, 0, 1) and top (1, 0, 0, 2.5) states
void RT_boundary(Fluid2d* fluids, Block2d) {
    Fluid2d bottom, top;
    const double b[4] = {2.0, 0.0, 0.0, 1.0}, t[4] = {1.0, 0.0, 0.0, 2.5};
    for (int v = 0; v < 4; ++v) {
        bottom.primvar[v] = b[v];
        top.primvar[v] = t[v];
    }
    record2(fluids, 0, HOS_BC_REFLECT, nullptr);
    record2(fluids, 1, HOS_BC_REFLECT, nullptr);
    record2(fluids, 2, HOS_BC_INFLOW, &bottom);
    record2(fluids, 3, HOS_BC_INFLOW, &top);
}

namespace {
void update2(Fluid2d* fluids, Block2d block, int stage, bool source) {
    Ctx2& c = live2(fluids, "Update");
    if (stage != c.next) stop(HOS_E_CONFIG, "wrong middle stage,pls check the time marching setting");
    if (is_using_df_factor && cellreconstruction_2D_normal == WENO5_AO_normal)
        stop(HOS_E_CONFIG, "WENO5_AO_normal with is_using_df_factor = true: the GPU path runs the DF variants while "
                           "the driver updates the DF indicators (assign WENO5_AO_with_df_normal / _tangent)");
    if (stage == 0) {
        int order = 0;
        const hos_params2d q = params2(block, &order);
        if (order != c.order || q.use_df != c.use_df) {
            // a driver may pick its reconstruction after Get_CFL (src/2Dproblem.cpp:133-137);
            // before the first stage the solver is rebuilt for it with the same dt
            if (c.stepped) stop(HOS_E_CONFIG, "the reconstruction order changed under a running solver");
            hos2d_destroy(c.h);
            c.h = nullptr;
            c.next = -1;
            Block2d b = block;
            create2(c, b, fluids);
            check2(hos2d_begin_step(c.h, c.tstop), "rebuild");  // the same dt: it depends on the state
            c.next = 0;
        }
    }
    {
        // the slots may switch between first order and WENO-AO from one step to the next
        int order = 0, fo = 0;
        const hos_params2d q = params2(block, &order, &fo);
        if (order != c.order || q.use_df != c.use_df)
            stop(HOS_E_CONFIG, "the reconstruction order changed under a running solver");
        check2(hos2d_set_reconstruction(c.h, fo ? HOS_RECON_FIRST_ORDER : HOS_RECON_WENO), "Update");
        check2(hos2d_set_source(c.h, source ? 1 : 0), "Update_with_source");
    }
    apply_boundaries2(c);
    check2(hos2d_stage(c.h, stage), "Update");
    c.stepped = true;
    c.next = stage + 1;
    if (!g_mirror) c.prim_last.clear();   // a later download converts the final state
    else if (c.next == block.stages - 1) {
        // the reference's Fluid2d::primvar after a step holds the state converted at the start
        // of the last stage (Convar_to_Primvar after its boundary fill): keep that state's
        // primitives for the copy back
        c.prim_last.resize(4 * (size_t)c.nx * c.ny);
        check2(hos2d_boundary(c.h), "Update");
        check2(hos2d_get_state(c.h, nullptr, c.prim_last.data(), nullptr, nullptr), "Update");
    }
    if (c.next == block.stages) {
        c.next = -1;
        double t = 0, dt = 0;
        const int st = hos2d_sync(c.h, &t, &dt);
        if (st == HOS_E_BLOWUP) blow_up(block.t);
        check2(st, "Update");
        if (g_mirror) download2(c, fluids);
    }
}
}  // namespace

// fused: the device updates the DF indicators at the end of each stage
void Update_alpha(Interface2d*, Interface2d*, Fluid2d* fluids, Block2d) { known2(fluids, "Update_alpha"); }

// the other methods' coefficient tables (src/time_advance.cpp:198-247); RK3 combines
// states in its update and sets none
void S1O1_2D(Block2d& block) {
    block.stages = 1;
    block.timecoefficient[0][0][0] = 1.0;
    block.timecoefficient[0][0][1] = 0.0;
}
void S1O2_2D(Block2d& block) {
    block.stages = 1;
    block.timecoefficient[0][0][0] = 1.0;
    block.timecoefficient[0][0][1] = 0.5;
}
void RK2_2D(Block2d& block) {
    block.stages = 2;
    block.timecoefficient[0][0][0] = 1.0;
    block.timecoefficient[1][0][0] = 0.5;
    block.timecoefficient[1][1][0] = 0.5;
}
void RK3_2D(Block2d& block) { block.stages = 3; }
void RK4_2D(Block2d& block) {
    block.stages = 4;
    block.timecoefficient[0][0][0] = 0.5;
    block.timecoefficient[1][1][0] = 0.5;
    block.timecoefficient[2][2][0] = 1.0;
    block.timecoefficient[3][0][0] = 1.0 / 6.0;
    block.timecoefficient[3][1][0] = 1.0 / 3.0;
    block.timecoefficient[3][2][0] = 1.0 / 3.0;
    block.timecoefficient[3][3][0] = 1.0 / 6.0;
}

// the two-stage fourth-order method: stage 1 at dt/2 with coefficients (1/2 of F, 1/8 of the
// flux time-derivative), stage 2 combining both stages (1/6, 1/3) (src/time_advance.cpp:221-230)
void S2O4_2D(Block2d& block) {
    block.stages = 2;
    block.timecoefficient[0][0][0] = 0.5;
    block.timecoefficient[0][0][1] = 1.0 / 8.0;
    block.timecoefficient[1][0][0] = 1.0;
    block.timecoefficient[1][1][0] = 0.0;
    block.timecoefficient[1][0][1] = 1.0 / 6.0;
    block.timecoefficient[1][1][1] = 1.0 / 3.0;
}

void Initial_stages(Block2d& block) {
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j)
            for (int k = 0; k < 2; ++k) block.timecoefficient[i][j][k] = 0.0;
    timecoe_list_2d(block);
}

// boundary slots: record the side's kind; the device fills the ghost cells in the stage
void free_boundary_left(Fluid2d* f, Block2d, Fluid2d) { record2(f, 0, HOS_BC_FREE, nullptr); }
void free_boundary_right(Fluid2d* f, Block2d, Fluid2d) { record2(f, 1, HOS_BC_FREE, nullptr); }
void free_boundary_down(Fluid2d* f, Block2d, Fluid2d) { record2(f, 2, HOS_BC_FREE, nullptr); }
void free_boundary_up(Fluid2d* f, Block2d, Fluid2d) { record2(f, 3, HOS_BC_FREE, nullptr); }
void periodic_boundary_left(Fluid2d* f, Block2d, Fluid2d) { record2(f, 0, HOS_BC_PERIODIC, nullptr); }
void periodic_boundary_right(Fluid2d* f, Block2d, Fluid2d) { record2(f, 1, HOS_BC_PERIODIC, nullptr); }
void periodic_boundary_down(Fluid2d* f, Block2d, Fluid2d) { record2(f, 2, HOS_BC_PERIODIC, nullptr); }
void periodic_boundary_up(Fluid2d* f, Block2d, Fluid2d) { record2(f, 3, HOS_BC_PERIODIC, nullptr); }
void reflection_boundary_left(Fluid2d* f, Block2d, Fluid2d) { record2(f, 0, HOS_BC_REFLECT, nullptr); }
void reflection_boundary_right(Fluid2d* f, Block2d, Fluid2d) { record2(f, 1, HOS_BC_REFLECT, nullptr); }
void reflection_boundary_down(Fluid2d* f, Block2d, Fluid2d) { record2(f, 2, HOS_BC_REFLECT, nullptr); }
void reflection_boundary_up(Fluid2d* f, Block2d, Fluid2d) { record2(f, 3, HOS_BC_REFLECT, nullptr); }
void inflow_boundary_left(Fluid2d* f, Block2d, Fluid2d v) { record2(f, 0, HOS_BC_INFLOW, &v); }
void inflow_boundary_right(Fluid2d* f, Block2d, Fluid2d v) { record2(f, 1, HOS_BC_INFLOW, &v); }
void inflow_boundary_up(Fluid2d* f, Block2d, Fluid2d v) { record2(f, 3, HOS_BC_INFLOW, &v); }
void noslip_adiabatic_boundary_left(Fluid2d* f, Block2d, Fluid2d v) { record2(f, 0, HOS_BC_NOSLIP, &v); }
void noslip_adiabatic_boundary_right(Fluid2d* f, Block2d, Fluid2d v) { record2(f, 1, HOS_BC_NOSLIP, &v); }
void noslip_adiabatic_boundary_down(Fluid2d* f, Block2d, Fluid2d v) { record2(f, 2, HOS_BC_NOSLIP, &v); }
void noslip_adiabatic_boundary_up(Fluid2d* f, Block2d, Fluid2d v) { record2(f, 3, HOS_BC_NOSLIP, &v); }

// reconstruction / flux slot values: identify the scheme; the work is fused in the stage
void First_order_normal(Interface2d&, Interface2d&, Interface2d&, Interface2d&, Fluid2d*, Block2d) { not_fused("First_order_normal"); }
void WENO5_AO_normal(Interface2d&, Interface2d&, Interface2d&, Interface2d&, Fluid2d*, Block2d) { not_fused("WENO5_AO_normal"); }
void WENO5_AO_with_df_normal(Interface2d&, Interface2d&, Interface2d&, Interface2d&, Fluid2d*, Block2d) { not_fused("WENO5_AO_with_df_normal"); }
void WENO7_AO_with_df_normal(Interface2d&, Interface2d&, Interface2d&, Interface2d&, Fluid2d*, Block2d) { not_fused("WENO7_AO_with_df_normal"); }
void WENO9_AO_with_df_normal(Interface2d&, Interface2d&, Interface2d&, Interface2d&, Fluid2d*, Block2d) { not_fused("WENO9_AO_with_df_normal"); }
void First_order_tangent(Interface2d*, Interface2d*, Interface2d*, Interface2d*, Fluid2d*, Block2d) { not_fused("First_order_tangent"); }
void WENO5_AO_tangent(Interface2d*, Interface2d*, Interface2d*, Interface2d*, Fluid2d*, Block2d) { not_fused("WENO5_AO_tangent"); }
void WENO5_AO_with_df_tangent(Interface2d*, Interface2d*, Interface2d*, Interface2d*, Fluid2d*, Block2d) { not_fused("WENO5_AO_with_df_tangent"); }
void WENO7_AO_with_df_tangent(Interface2d*, Interface2d*, Interface2d*, Interface2d*, Fluid2d*, Block2d) { not_fused("WENO7_AO_with_df_tangent"); }
void WENO9_AO_with_df_tangent(Interface2d*, Interface2d*, Interface2d*, Interface2d*, Fluid2d*, Block2d) { not_fused("WENO9_AO_with_df_tangent"); }
void Center_do_nothing_normal(Interface2d*, Interface2d*, Fluid2d*, Block2d) {}
void Center_all_collision_multi(Interface2d*, Interface2d*, Fluid2d*, Block2d) { not_fused("Center_all_collision_multi"); }
void GKS2D_smooth(Flux2d&, Recon2d&, double) { not_fused("GKS2D_smooth"); }
void GKS2D(Flux2d&, Recon2d&, double) { not_fused("GKS2D"); }
void LF2D(Flux2d&, Recon2d&, double) { not_fused("LF2D"); }

// ======================================= 1D API =======================================

double Get_CFL(Block1d& block, Fluid1d* fluids, double tstop) {
    Ctx1& c = g_ctx1[fluids];
    if (c.next >= 0) stop(HOS_E_CONFIG, "Get_CFL called inside a time step");
    if (!c.h) create1(c, block, fluids);
    else if (block.nx != c.nx || block.CFL != c.cfl)
        stop(HOS_E_CONFIG, "the Block1d changed under a running solver: call hos_ref_release first");
    check1(hos1d_begin_step(c.h, tstop), "Get_CFL");
    double t = 0, dt = 0;
    const int st = hos1d_sync(c.h, &t, &dt);
    if (st == HOS_E_BLOWUP) blow_up(block.t);
    check1(st, "Get_CFL");
    c.next = 0;
    return dt;
}

void CopyFluid_new_to_old(Fluid1d* fluids, Block1d block) {
    if (!g_mirror) return;
    for (int i = block.ghost; i < block.ghost + block.nodex; ++i)
        for (int v = 0; v < 3; ++v) fluids[i].convar_old[v] = fluids[i].convar[v];
}

void Reconstruction_within_cell(Interface1d*, Fluid1d* fluids, Block1d) { live1(fluids, "Reconstruction_within_cell"); }
void Reconstruction_forg0(Interface1d*, Fluid1d* fluids, Block1d) { live1(fluids, "Reconstruction_forg0"); }

void Calculate_flux(Flux1d**, Interface1d*, Block1d& block, int stage) {
    if (stage < 0 || stage >= block.stages)
        stop(HOS_E_CONFIG, "wrong middle stage,pls check the time marching setting");
}

void Update(Fluid1d* fluids, Flux1d**, Block1d block, int stage) {
    Ctx1& c = live1(fluids, "Update");
    if (stage != c.next) stop(HOS_E_CONFIG, "wrong middle stage,pls check the time marching setting");
    if (stage == 0) {
        // the device switches WENO5_AO -> WENO5_AO_with_DF after its first step (df_mode 2)
        bool df = false;
        const int order = order1(cellreconstruction, &df);
        const bool want_df = c.df_mode == 1 || (c.df_mode == 2 && c.steps > 0);
        if (order != c.order || df != want_df)
            stop(HOS_E_CONFIG, "cellreconstruction changed in a way the GPU solver does not follow");
    }
    if ((c.pend_mask & 3u) != 3u) stop(HOS_E_CONFIG, "call both boundary functions before Update in each stage");
    for (int s = 0; s < 2; ++s)
        if (c.pend[s].kind < 0) stop(HOS_E_CONFIG, "the GPU path provides free, periodic and reflective 1D boundaries");
    if (c.pend[0].kind != c.cur[0].kind || c.pend[1].kind != c.cur[1].kind) {
        const int kinds[2] = {c.pend[0].kind, c.pend[1].kind};
        check1(hos1d_set_boundary(c.h, kinds), "boundary");
        c.cur[0] = c.pend[0];
        c.cur[1] = c.pend[1];
    }
    c.pend_mask = 0;
    check1(hos1d_stage(c.h, stage), "Update");
    c.next = stage + 1;
    if (c.next == block.stages) {
        c.next = -1;
        ++c.steps;
        double t = 0, dt = 0;
        const int st = hos1d_sync(c.h, &t, &dt);
        if (st == HOS_E_BLOWUP) blow_up(block.t);
        check1(st, "Update");
        if (g_mirror) download1(c, fluids);
    }
}

void Update_alpha(Interface1d*, Fluid1d* fluids, Block1d) { known1(fluids, "Update_alpha"); }

void S1O1(Block1d& block) { block.stages = 1; }
void S1O2(Block1d& block) { block.stages = 1; }
void RK2(Block1d& block) { block.stages = 2; }
void RK3(Block1d& block) { block.stages = 3; }
void RK4(Block1d& block) { block.stages = 4; }

void S2O4(Block1d& block) {
    block.stages = 2;
    block.timecoefficient[0][0][0] = 0.5;
    block.timecoefficient[0][0][1] = 1.0 / 8.0;
    block.timecoefficient[1][0][0] = 1.0;
    block.timecoefficient[1][1][0] = 0.0;
    block.timecoefficient[1][0][1] = 1.0 / 6.0;
    block.timecoefficient[1][1][1] = 1.0 / 3.0;
}

void Initial_stages(Block1d& block) {
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j)
            for (int k = 0; k < 2; ++k) block.timecoefficient[i][j][k] = 0.0;
    timecoe_list(block);
}

void free_boundary_left(Fluid1d* f, Block1d, Fluid1d) { record1(f, 0, HOS_BC_FREE); }
void free_boundary_right(Fluid1d* f, Block1d, Fluid1d) { record1(f, 1, HOS_BC_FREE); }
void reflection_boundary_left(Fluid1d* f, Block1d, Fluid1d) { record1(f, 0, HOS_BC_REFLECT); }
void reflection_boundary_right(Fluid1d* f, Block1d, Fluid1d) { record1(f, 1, HOS_BC_REFLECT); }
void periodic_boundary_left(Fluid1d* f, Block1d, Fluid1d) { record1(f, 0, HOS_BC_PERIODIC); }
void periodic_boundary_right(Fluid1d* f, Block1d, Fluid1d) { record1(f, 1, HOS_BC_PERIODIC); }

void Vanleer(Point1d&, Point1d&, Fluid1d*, Block1d) { not_fused("Vanleer"); }
void WENO5_AO(Point1d&, Point1d&, Fluid1d*, Block1d) { not_fused("WENO5_AO"); }
void WENO5_AO_with_DF(Point1d&, Point1d&, Fluid1d*, Block1d) { not_fused("WENO5_AO_with_DF"); }
void WENO7_AO_with_DF(Point1d&, Point1d&, Fluid1d*, Block1d) { not_fused("WENO7_AO_with_DF"); }
void WENO9_AO_with_DF(Point1d&, Point1d&, Fluid1d*, Block1d) { not_fused("WENO9_AO_with_DF"); }
void Center_collision(Interface1d&, Fluid1d*) { not_fused("Center_collision"); }
void GKS(Flux1d&, Interface1d&, double) { not_fused("GKS"); }
void LF(Flux1d&, Interface1d&, double) { not_fused("LF"); }

// ======================================= controls =======================================

extern "C" {

void hos_ref_set_precision(int precision) { g_precision = precision == HOS_FP32 ? HOS_FP32 : HOS_FP64; }
void hos_ref_set_mirror(int on) { g_mirror = on != 0; }
void hos_ref_set_error_mode(int mode) { g_mode = mode == HOS_REF_THROW ? HOS_REF_THROW : HOS_REF_EXIT; }

int hos_ref_set_wedge2d(const Fluid2d* fluids, double x0, double top_speed, const double* post_prim,
                        const double* pre_prim) {
    if (!fluids || !post_prim || !pre_prim) return HOS_E_ARG;
    Ctx2& c = ctx2(fluids);
    if (c.h) return HOS_E_CONFIG;   // declare before the first step
    c.wedge = true;
    c.wx0 = x0;
    c.wspeed = top_speed;
    for (int v = 0; v < 4; ++v) {
        c.wpost[v] = post_prim[v];
        c.wpre[v] = pre_prim[v];
    }
    return HOS_OK;
}

int hos_ref_download2d(Fluid2d* fluids, Block2d) {
    auto it = g_ctx2.find(fluids);
    if (it == g_ctx2.end() || !it->second.h) return HOS_E_ARG;
    download2(it->second, fluids);
    return HOS_OK;
}

int hos_ref_upload2d(Fluid2d* fluids, Block2d block) {
    auto it = g_ctx2.find(fluids);
    if (it == g_ctx2.end() || !it->second.h) return HOS_OK;   // the next Get_CFL uploads
    if (it->second.next >= 0) return HOS_E_CONFIG;
    upload2(it->second, fluids, block.t);
    return HOS_OK;
}

int hos_ref_download1d(Fluid1d* fluids, Block1d) {
    auto it = g_ctx1.find(fluids);
    if (it == g_ctx1.end() || !it->second.h) return HOS_E_ARG;
    download1(it->second, fluids);
    return HOS_OK;
}

int hos_ref_upload1d(Fluid1d* fluids, Block1d block) {
    auto it = g_ctx1.find(fluids);
    if (it == g_ctx1.end() || !it->second.h) return HOS_OK;
    if (it->second.next >= 0) return HOS_E_CONFIG;
    upload1(it->second, fluids, block.t);
    return HOS_OK;
}

void hos_ref_release(const void* fluids) {
    auto a = g_ctx2.find(fluids);
    if (a != g_ctx2.end()) {
        if (a->second.h) hos2d_destroy(a->second.h);
        g_ctx2.erase(a);
    }
    auto b = g_ctx1.find(fluids);
    if (b != g_ctx1.end()) {
        if (b->second.h) hos1d_destroy(b->second.h);
        g_ctx1.erase(b);
    }
}

hos_solver2d* hos_ref_solver2d(const Fluid2d* fluids) {
    auto it = g_ctx2.find(fluids);
    return it == g_ctx2.end() ? nullptr : it->second.h;
}

hos_solver1d* hos_ref_solver1d(const Fluid1d* fluids) {
    auto it = g_ctx1.find(fluids);
    return it == g_ctx1.end() ? nullptr : it->second.h;
}

}  // extern "C"
