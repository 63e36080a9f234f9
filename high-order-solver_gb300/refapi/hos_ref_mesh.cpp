// hos_ref_mesh.cpp -- the data-model half of the reference's function-level API: the globals
// its drivers set, Gauss points, the Fluid/Interface/Flux allocators and the uniform-mesh
// geometry (src/basic_function.cpp:3-13, 1262-1560; src/fluid_mesh.cpp:3-45).  These run on
// the host, once per problem, exactly as in the reference: they fill the driver's arrays; the
// per-step work is in hos_ref_path.cpp.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "hos_ref_api.h"

// globals with the reference's initial values (src/basic_function.cpp:3-13, src/fluid_mesh.cpp:3-5)
int K = 0;
double Gamma = 2.0 / (K + 2) + 1.0;
double T_inf = 285;
double R_gas = 8.31441 / (28.959e-3);
double Mu = -1.0;
double Nu = -1.0;
double c1_euler = -1.0;
double c2_euler = -1.0;
bool is_Prandtl_fix = false;
double Pr = 1.0;
TAU_TYPE tau_type = Euler;
int gausspoint = 0;
double* gauss_loc = nullptr;
double* gauss_weight = nullptr;

// Gauss nodes on [-1, 1] and weights summing to 1 per gausspoint (SetGuassPoint,
// src/fluid_mesh.cpp:9-45): Gauss-Legendre for 1-3 points, Gauss-Lobatto for 4.
void SetGuassPoint() {
    if (gausspoint < 1 || gausspoint > 4) {
        std::printf("no gausspoint specify\n");
        std::exit(0);
    }
    delete[] gauss_loc;
    delete[] gauss_weight;
    gauss_loc = new double[gausspoint];
    gauss_weight = new double[gausspoint];
    switch (gausspoint) {
        case 1:
            gauss_loc[0] = 0.0;
            gauss_weight[0] = 1.0;
            break;
        case 2:
            gauss_loc[0] = -std::sqrt(1.0 / 3.0);
            gauss_loc[1] = -gauss_loc[0];
            gauss_weight[0] = gauss_weight[1] = 0.5;
            break;
        case 3:
            gauss_loc[0] = 0.0;
            gauss_loc[1] = std::sqrt(3.0 / 5.0);
            gauss_loc[2] = -gauss_loc[1];
            gauss_weight[0] = 4.0 / 9.0;
            gauss_weight[1] = gauss_weight[2] = 0.5 - 0.5 * gauss_weight[0];
            break;
        default:
            gauss_loc[0] = -1.0;
            gauss_loc[1] = 1.0;
            gauss_loc[2] = -std::sqrt(5.0) / 5.0;
            gauss_loc[3] = -gauss_loc[2];
            gauss_weight[0] = gauss_weight[1] = 1.0 / 12.0;
            gauss_weight[2] = gauss_weight[3] = 5.0 / 12.0;
    }
}

// ---------------- 1D ----------------

Flux1d** Setflux_array(Block1d block) {
    Flux1d** fx = new Flux1d*[block.nx + 1];
    for (int i = 0; i <= block.nx; ++i) {
        fx[i] = new Flux1d[block.stages];
        for (int s = 0; s < block.stages; ++s)
            for (int v = 0; v < 3; ++v) fx[i][s].f[v] = fx[i][s].derf[v] = 0.0;
    }
    return fx;
}

void SetUniformMesh(Block1d block, Fluid1d* fluids, Interface1d* interfaces, Flux1d** fluxes) {
    for (int i = 0; i < block.nx; ++i) {
        fluids[i].dx = block.dx;
        fluids[i].cx = block.left + (i + 0.5 - block.ghost) * block.dx;
    }
    for (int i = 0; i <= block.nx; ++i) {
        Interface1d& f = interfaces[i];
        f.x = block.left + (i - block.ghost) * block.dx;
        f.left.x = f.right.x = f.center.x = f.x;
        f.flux = fluxes[i];
    }
}

// ---------------- 2D ----------------

Fluid2d* Setfluid(Block2d& block) {
    Fluid2d* f = new Fluid2d[(size_t)block.nx * block.ny];
    for (int i = 0; i < block.nx; ++i)
        for (int j = 0; j < block.ny; ++j) {
            f[(size_t)i * block.ny + j].xindex = i;
            f[(size_t)i * block.ny + j].yindex = j;
        }
    return f;
}

Interface2d* Setinterface_array(Block2d block) {
    const size_t n = (size_t)(block.nx + 1) * (block.ny + 1);
    Interface2d* f = new Interface2d[n];
    for (size_t k = 0; k < n; ++k)
        for (int v = 0; v < 4; ++v) {
            Recon2d& r = f[k].line;
            r.left.der1x[v] = r.left.der1y[v] = 0.0;
            r.right.der1x[v] = r.right.der1y[v] = 0.0;
            r.center.der1x[v] = r.center.der1y[v] = 0.0;
        }
    return f;
}

Flux2d_gauss** Setflux_gauss_array(Block2d block) {
    const size_t n = (size_t)(block.nx + 1) * (block.ny + 1);
    const int gp = gausspoint == 0 ? 1 : gausspoint;
    Flux2d_gauss** f = new Flux2d_gauss*[n];
    for (size_t k = 0; k < n; ++k) {
        f[k] = new Flux2d_gauss[block.stages];
        for (int s = 0; s < block.stages; ++s) {
            f[k][s].gauss = new Flux2d[gp];
            for (int g = 0; g < gp; ++g)
                for (int v = 0; v < 4; ++v) f[k][s].gauss[g].f[v] = f[k][s].gauss[g].derf[v] = 0.0;
        }
    }
    return f;
}

namespace {

void face_geometry(Interface2d& f, Flux2d_gauss* flux, int stages, double x, double y, double length, double nx_,
                   double ny_, bool xface) {
    f.x = x;
    f.y = y;
    f.length = length;
    f.normal[0] = nx_;
    f.normal[1] = ny_;
    f.line.x = x;
    f.line.y = y;
    f.line.normal[0] = nx_;
    f.line.normal[1] = ny_;
    f.gauss = new Recon2d[gausspoint];
    const int gp = gausspoint == 0 ? 1 : gausspoint;
    for (int s = 0; s < stages; ++s)
        for (int g = 0; g < gp; ++g) {
            flux[s].gauss[g].normal[0] = nx_;
            flux[s].gauss[g].normal[1] = ny_;
            flux[s].gauss[g].length = length;
        }
    // Gauss point positions along the face; the left/right/centre points hold the offset
    // along the face in their tangential coordinate
    for (int g = 0; g < gausspoint; ++g) {
        Recon2d& r = f.gauss[g];
        const double off = gauss_loc[g] * 0.5 * length;
        r.x = xface ? x : x + off;
        r.y = xface ? y + off : y;
        r.normal[0] = nx_;
        r.normal[1] = ny_;
        Point2d* pts[3] = {&r.left, &r.right, &r.center};
        for (Point2d* p : pts) {
            if (xface) p->y = gauss_loc[g] * length / 2.0;
            else p->x = gauss_loc[g] * length / 2.0;
        }
    }
}

}  // namespace

void SetUniformMesh(Block2d& block, Fluid2d* fluids, Interface2d* xinterfaces, Interface2d* yinterfaces,
                    Flux2d_gauss** xfluxes, Flux2d_gauss** yfluxes) {
    block.dx = (block.right - block.left) / block.nodex;
    block.dy = (block.up - block.down) / block.nodey;
    block.overdx = 1 / block.dx;
    block.overdy = 1 / block.dy;
    block.xcell_begin = block.ghost;
    block.xcell_end = block.ghost + block.nodex - 1;
    block.ycell_begin = block.ghost;
    block.ycell_end = block.ghost + block.nodey - 1;
    block.xinterface_begin_n = block.ghost;
    block.xinterface_end_n = block.ghost + block.nodex;
    block.xinterface_begin_t = block.ghost;
    block.xinterface_end_t = block.ghost + block.nodex - 1;
    block.yinterface_begin_n = block.ghost;
    block.yinterface_end_n = block.ghost + block.nodey;
    block.yinterface_begin_t = block.ghost;
    block.yinterface_end_t = block.ghost + block.nodey - 1;
    const double dx = block.dx, dy = block.dy;
    for (int i = 0; i < block.nx; ++i)
        for (int j = 0; j < block.ny; ++j) {
            Fluid2d& c = fluids[(size_t)i * block.ny + j];
            c.dx = dx;
            c.dy = dy;
            c.coordx = block.left + (i + 0.5 - block.ghost) * dx;
            c.coordy = block.down + (j + 0.5 - block.ghost) * dy;
            c.area = dx * dy;
            const double x0 = block.left + (i - block.ghost) * dx, x1 = block.left + (i + 1 - block.ghost) * dx;
            const double y0 = block.down + (j - block.ghost) * dy, y1 = block.down + (j + 1 - block.ghost) * dy;
            const double nodes[8] = {x0, y0, x1, y0, x1, y1, x0, y1};   // counter-clockwise corners
            for (int k = 0; k < 8; ++k) c.node[k] = nodes[k];
        }
    for (int i = 0; i <= block.nx; ++i)
        for (int j = 0; j <= block.ny; ++j) {
            const size_t k = (size_t)i * (block.ny + 1) + j;
            face_geometry(xinterfaces[k], xfluxes[k], block.stages, block.left + (i - block.ghost) * dx,
                          block.down + (j - block.ghost + 0.5) * dy, dy, 1.0, 0.0, true);
            face_geometry(yinterfaces[k], yfluxes[k], block.stages, block.left + (i - block.ghost + 0.5) * dx,
                          block.down + (j - block.ghost) * dy, dx, 0.0, 1.0, false);
        }
}
