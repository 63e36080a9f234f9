// ref_driver3d.cpp -- non-interactive driver of the UNMODIFIED reference sources for the 3D
// step (CubicTube's loop, src/3Dproblem.cpp:125-157).
//
// TEST INFRASTRUCTURE ONLY (built into oracle/_ref/, never shipped, never linked by the
// product).  It sets the globals and the Block3d the way CubicTube does
// (src/3Dproblem.cpp:3-104), allocates through the reference's own Setfluid_array /
// Setinterface_array / Setflux_gauss_array / SetUniformMesh, and calls the reference's stage
// functions in the loop's order.  One thing is added: the reference never allocates the
// Gauss-point array Interface3d::gauss (Allocate_reconstruction_variable_along_interface,
// src/basic_function.cpp:1896-1904, allocates only `line`) although the point reconstruction
// and the flux write and read it (src/reconstruction.cpp:4153-4159, src/flux_function.cpp:
// 772-806), so its 3D path faults at the first stage.  The harness allocates it, 4 points per
// face, value-initialised (order_reduce = false, as the lines start), after SetUniformMesh.
#include "3Dproblem.h"

#include <cstring>
#include <vector>

#include "oracle_api.h"

namespace {
Block3d g_block;
Fluid3d* g_fluids = nullptr;
Interface3d* g_if[3] = {nullptr, nullptr, nullptr};
Flux3d_gauss** g_fl[3] = {nullptr, nullptr, nullptr};
Fluid3d g_bcvalue[6];

size_t ncell() { return (size_t)g_block.nx * g_block.ny * g_block.nz; }
size_t nface() { return (size_t)(g_block.nx + 1) * (g_block.ny + 1) * (g_block.nz + 1); }
}  // namespace

extern "C" {

int ref3d_init(const hos3d_params* p) {
    for (int s = 0; s < 6; ++s)
        if (p->bc[s] != HOS_BC_FREE) return 2;   // the reference's 3D boundaries are free ones
    if (p->prandtl_fix) return 2;               // GKS3D has no Prandtl-number correction
    Block3d block;
    std::memset(&block, 0, sizeof block);
    block.uniform = true;
    block.nodex = p->nodex;
    block.nodey = p->nodey;
    block.nodez = p->nodez;
    block.ghost = p->ghost;
    block.CFL = p->cfl;
    K = p->K;
    Gamma = p->gamma;
    gks3dsolver = gks2nd_3d;
    tau_type = p->tau_type == 1 ? NS : Euler;
    Mu = p->mu;
    c1_euler = p->c1_euler;
    c2_euler = p->c2_euler;
    gausspoint = 4;
    SetGuassPoint_3D();
    reconstruction_variable = p->characteristic ? characteristic : conservative;
    wenotype = wenoz;
    cellreconstruction_3D_of_face_value = WENO5_AO_splitting_3d;
    cellreconstruction_3D_of_line_value = WENO5_AO_of_line_value;
    cellreconstruction_3D_of_point_value = WENO5_AO_of_point_value;
    g0reconstruction_3D_of_face_value = Do_nothing_splitting_3d;
    g0reconstruction_3D_of_line_value = Do_nothing_reconstruction_of_line_value;
    g0reconstruction_3D_of_point_value = Do_nothing_reconstruction_of_point_value;
    g0type = all_collisionn;
    flux_function_3d = GKS3D;
    timecoe_list_3d = S2O4_3D;
    Initial_stages(block);
    block.nx = block.nodex + 2 * block.ghost;
    block.ny = block.nodey + 2 * block.ghost;
    block.nz = block.nodez + 2 * block.ghost;
    g_fluids = Setfluid_array(block);
    for (int d = 0; d < 3; ++d) {
        g_if[d] = Setinterface_array(block);
        g_fl[d] = Setflux_gauss_array(block);
    }
    block.left = p->left;
    block.right = p->right;
    block.down = p->down;
    block.up = p->up;
    block.back = p->back;
    block.front = p->front;
    block.dx = (block.right - block.left) / block.nodex;
    block.dy = (block.up - block.down) / block.nodey;
    block.dz = (block.front - block.back) / block.nodez;
    block.xarea = block.dy * block.dz;
    block.yarea = block.dx * block.dz;
    block.zarea = block.dx * block.dy;
    block.overdx = 1 / block.dx;
    block.overdy = 1 / block.dy;
    block.overdz = 1 / block.dz;
    SetUniformMesh(block, g_fluids, g_if[0], g_if[1], g_if[2]);
    g_block = block;
    for (int d = 0; d < 3; ++d)
        for (size_t f = 0; f < nface(); ++f) g_if[d][f].gauss = new Recon3d[gausspoint]();
    return 0;
}

void ref3d_set_threads(int n) { omp_set_num_threads(n); }

void ref3d_set_state(const double* convar, const double* primvar) {
    for (size_t c = 0; c < ncell(); ++c) {
        for (int v = 0; v < 5; ++v) g_fluids[c].convar[v] = convar[5 * c + v];
        if (primvar)
            for (int v = 0; v < 5; ++v) g_fluids[c].primvar[v] = primvar[5 * c + v];
        else
            Convar_to_primvar_3D(g_fluids[c].primvar, g_fluids[c].convar);
    }
}

void ref3d_get_state(double* convar, double* primvar) {
    for (size_t c = 0; c < ncell(); ++c)
        for (int v = 0; v < 5; ++v) {
            if (convar) convar[5 * c + v] = g_fluids[c].convar[v];
            if (primvar) primvar[5 * c + v] = g_fluids[c].primvar[v];
        }
}

double ref3d_begin_step(double tstop, double t) {
    g_block.t = t;
    CopyFluid_new_to_old(g_fluids, g_block);
    return Get_CFL(g_block, g_fluids, tstop);
}

int ref3d_stage(int stage, double dt) {
    g_block.dt = dt;
    free_boundary_xleft(g_fluids, g_block, g_bcvalue[0]);
    free_boundary_xright(g_fluids, g_block, g_bcvalue[1]);
    free_boundary_yleft(g_fluids, g_block, g_bcvalue[2]);
    free_boundary_yright(g_fluids, g_block, g_bcvalue[3]);
    free_boundary_zleft(g_fluids, g_block, g_bcvalue[4]);
    free_boundary_zright(g_fluids, g_block, g_bcvalue[5]);
    // Convar_to_primvar exits on a blow-up; the harness reports a status first
    for (size_t c = 0; c < ncell(); ++c) {
        double pr[5];
        Convar_to_primvar_3D(pr, g_fluids[c].convar);
        if (pr[0] < 0 || pr[4] < 0 || pr[0] != pr[0] || pr[4] != pr[4]) return 1;
    }
    Convar_to_primvar(g_fluids, g_block);
    Reconstruction_within_cell(g_if[0], g_if[1], g_if[2], g_fluids, g_block);
    Reconstruction_forg0(g_if[0], g_if[1], g_if[2], g_fluids, g_block);
    Calculate_flux(g_fl[0], g_fl[1], g_fl[2], g_if[0], g_if[1], g_if[2], g_block, stage);
    Update_gauss(g_fluids, g_fl[0], g_fl[1], g_fl[2], g_block, stage);
    return 0;
}

int ref3d_step(double tstop, double t, double* dt_out) {
    const double dt = ref3d_begin_step(tstop, t);
    if (dt_out) *dt_out = dt;
    for (int s = 0; s < g_block.stages; ++s) {
        const int st = ref3d_stage(s, dt);
        if (st) return st;
    }
    g_block.step++;
    return 0;
}

// per interior face of direction dir, the stage fluxes summed over the 4 Gauss points with
// weight 1/4, in the face frame, laid out as oracle3d_get_flux: [face][stage][f 5, derf 5],
// faces ordered (normal, t1, t2) with x faces (i, j, k), y faces (j, nx-1-i, k), z faces
// (k, j, nx-1-i) over the interior faces
void ref3d_get_flux(int dir, double* out) {
    const Block3d& b = g_block;
    const int g = b.ghost;
    const int n0 = dir == 0 ? b.nx : dir == 1 ? b.ny : b.nz;
    const int n1 = dir == 0 ? b.ny : dir == 1 ? b.nx : b.ny;
    const int n2 = dir == 0 ? b.nz : dir == 1 ? b.nz : b.nx;
    const int nn = n0 - 2 * g + 1, m1 = n1 - 2 * g, m2 = n2 - 2 * g;
    for (int a = 0; a < nn; ++a)
        for (int p = 0; p < m1; ++p)
            for (int q = 0; q < m2; ++q) {
                const int A = a + g, B = p + g, C = q + g;
                int i, j, k;
                if (dir == 0) { i = A; j = B; k = C; }
                else if (dir == 1) { i = b.nx - 1 - B; j = A; k = C; }
                else { i = b.nx - 1 - C; j = B; k = A; }
                const size_t idx = ((size_t)i * (b.ny + 1) + j) * (b.nz + 1) + k;
                const size_t face = ((size_t)a * m1 + p) * m2 + q;
                for (int st = 0; st < 2; ++st) {
                    double acc[10] = {0};
                    for (int m = 0; m < gausspoint; ++m)
                        for (int v = 0; v < 5; ++v) {
                            acc[v] += 0.25 * g_fl[dir][idx][st].gauss[m].f[v];
                            acc[5 + v] += 0.25 * g_fl[dir][idx][st].gauss[m].derf[v];
                        }
                    for (int v = 0; v < 10; ++v) out[(face * 2 + st) * 10 + v] = acc[v];
                }
            }
}

// number of line and Gauss-point reconstructions whose order-reduction flag is set (the
// reference never clears them once set, src/reconstruction.cpp:4124-4132, 4380-4384)
long long ref3d_reduced_count(void) {
    long long n = 0;
    for (int d = 0; d < 3; ++d)
        for (size_t f = 0; f < nface(); ++f) {
            for (int m = 0; m < 2; ++m) n += g_if[d][f].line[m].order_reduce ? 1 : 0;
            for (int m = 0; m < gausspoint; ++m) n += g_if[d][f].gauss[m].order_reduce ? 1 : 0;
        }
    return n;
}

}  // extern "C"
