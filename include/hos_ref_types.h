/*
 * hos_ref_types.h -- the 1D/2D data model of XJTUZhangHong/high-order-solver
 * (include/fluid_mesh.h:8-222 and the enums/function-pointer types of include/reconstruction.h,
 * include/flux_function.h, include/time_advance.h, include/boundary_condition.h,
 * include/basic_function.h), declared with the same class names, member names, member
 * order and member types.
 *
 * Why these declarations repeat the reference's: the C++ layer in libhos_ref.so exports the
 * reference's hot-path functions under their C++ names (Reconstruction_within_cell(Interface2d*,
 * ...), Update(Fluid2d*, Flux2d_gauss**, ...), ...).  A driver compiled against the reference's
 * own headers links to it only if the mangled names (class names) and the object layouts
 * (member order and types) are identical, so that `fluids[i*ny+j].convar[v]` addresses the same
 * bytes on both sides.  Only the 1D and 2D classes the hot path touches are declared here.
 */
#ifndef HOS_REF_TYPES_H
#define HOS_REF_TYPES_H

#include <string>

/* ---------------- one-dimensional problem ---------------- */
class Block1d {
public:
    int ghost;
    int nodex;
    int nx;
    int nodex_begin;
    int nodex_end;
    double dx;
    double left;
    double right;
    int stages;
    double timecoefficient[5][5][2];
    double t;
    double CFL;
    double dt;
    int step;
};

class Fluid1d {
public:
    double primvar[3];
    double convar[3];
    double convar_old[3];
    double convar_stage1[3];
    double convar_stage2[3];
    double cx;
    double dx;
    double alpha = 0.0;
};

class Point1d {
public:
    double convar[3];
    double convar_old[3];
    double der1[3];
    double x;
};

class Flux1d {
public:
    double F[3];
    double f[3];
    double derf[4];
};

class Interface1d {
public:
    Point1d left;
    Point1d center;
    Point1d right;
    Flux1d* flux;
    double x;
};

/* ---------------- two-dimensional problem ---------------- */
class Block2d {
public:
    int index;
    bool uniform;
    int ghost;
    int nodex;
    int nodey;
    int nx;
    int ny;
    int xcell_begin;
    int xcell_end;
    int ycell_begin;
    int ycell_end;
    int xinterface_begin_n;
    int xinterface_begin_t;
    int xinterface_end_n;
    int xinterface_end_t;
    int yinterface_begin_n;
    int yinterface_begin_t;
    int yinterface_end_n;
    int yinterface_end_t;
    double dx;
    double dy;
    double overdx;
    double overdy;
    double left;
    double right;
    double down;
    double up;
    int stages;
    double timecoefficient[5][5][2];
    double t;
    double CFL;
    double dt;
    int step;
    double T;
    int outputperstep;
};

class Point2d {
public:
    double convar[4];
    double primvar[4];
    double der1x[4];
    double der1y[4];
    double x;
    double y;
    double normal[2];
    bool is_reduce_order;
};

class Fluid2d {
public:
    double primvar[4];
    double exact;
    double convar[4];
    double convar_old[4];
    double convar_stage1[4];
    double convar_stage2[2];
    double res[4];
    double xindex;
    double yindex;
    double coordx;
    double coordy;
    double dx;
    double dy;
    double area;
    bool is_hweno;
    double node[8];
    bool boundary;
    double alpha_x = 0.0;
    double alpha_y = 0.0;
    std::string direction;
    bool is_left = false;
    double Sw1[2][4];
    double Lw1[2][4];
    double derSw1[2][4];
    double derLw1[2][4];
};

class Flux2d {
public:
    double x[4];
    double f[4];
    double derf[4];
    double length;
    double normal[2];
};

class Recon2d {
public:
    Point2d left;
    Point2d center;
    Point2d right;
    double x;
    double y;
    double normal[2];
};

class Interface2d {
public:
    Recon2d line;
    Recon2d* gauss;
    double x;
    double y;
    double normal[2];
    double length;
};

class Flux2d_gauss {
public:
    Flux2d* gauss;
};

/* ---------------- configuration enums and function-pointer slots ---------------- */
enum TAU_TYPE { Euler, NS };                                               /* basic_function.h */
enum Reconstruction_variable { conservative, characteristic };             /* reconstruction.h */
enum WENOtype { linear, wenojs, wenoz };
enum GKS1d_type { nothing, kfvs1st, kfvs2nd, gks1st, gks2nd, pp_gks };     /* flux_function.h */
enum GKS2d_type { nothing_2d, kfvs1st_2d, kfvs2nd_2d, gks1st_2d, gks2nd_2d, pp_gks_2d };
enum G0_construct_type { collisionn, collisionnless, all_collisionn };

typedef void (*Reconstruction_within_Cell)(Point1d& left, Point1d& right, Fluid1d* fluids, Block1d block);
typedef void (*Reconstruction_forG0)(Interface1d& interfaces, Fluid1d* fluids);
typedef void (*Reconstruction_within_Cell_2D_normal)(Interface2d& left, Interface2d& right, Interface2d& down,
                                                     Interface2d& up, Fluid2d* fluids, Block2d block);
typedef void (*Reconstruction_within_Cell_2D_tangent)(Interface2d* left, Interface2d* right, Interface2d* down,
                                                      Interface2d* up, Fluid2d* fluids, Block2d block);
typedef void (*Reconstruction_forG0_2D_normal)(Interface2d* xinterfaces, Interface2d* yinterfaces, Fluid2d* fluids,
                                               Block2d block);
typedef void (*Reconstruction_forG0_2D_tangent)(Interface2d* xinterfaces, Interface2d* yinterfaces, Fluid2d* fluids,
                                                Block2d block);
typedef void (*Flux_function)(Flux1d& flux, Interface1d& interface, double dt);
typedef void (*Flux_function_2d)(Flux2d& flux, Recon2d& re, double dt);
typedef void (*TimeMarchingCoefficient)(Block1d& block);
typedef void (*TimeMarchingCoefficient_2d)(Block2d& block);
typedef void (*BoundaryCondition)(Fluid1d* fluids, Block1d block, Fluid1d bcvalue);
typedef void (*BoundaryCondition2d)(Fluid2d* fluids, Block2d block, Fluid2d bcvalue);

#endif /* HOS_REF_TYPES_H */
