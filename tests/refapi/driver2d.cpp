// driver2d.cpp -- a 2D problem driver written against the reference's own function-level API,
// following the loop of PlanarShock (src/2Dproblem.cpp:3-159) without its console prompts.
// Built two ways by the tests: against libhos_ref.so (the GPU path, include/hos_ref_api.h)
// and, with -DHOS_DRIVER_WITH_REFERENCE, against the reference's own sources, so both runs
// execute this same source.
//
//   driver2d <config.txt> <state_in.bin> <state_out.bin>
//
// config.txt: "key value..." lines (nodex nodey ghost order characteristic K gamma c1 c2 cfl
// left right down up bc (4 names) bcprim (side r u v p) steps tstop precision mirror, and
// optionally first_order_steps: steps that start with First_order_normal / _tangent, as the
// reference's drivers do at step 0 when is_using_df_factor is set, src/2Dproblem.cpp:733-745;
// tau_type (1: NS), mu, nu, prandtl_fix, pr: the collision-time globals; bc names may be
// noslip, whose wall velocity comes from the side's bcprim entry; source 1: the RT_instability
// loop, RT_boundary and Update_with_source, src/2Dproblem.cpp:746-763; df 0: the drivers'
// default with is_using_df_factor = false, the slots WENO5_AO_normal / WENO5_AO_tangent and
// the weights "wenotype z|js|linear", src/2Dproblem.cpp:35-38, 132-136).
// state_in.bin: convar then primvar, [nx*ny][4] doubles each.  state_out.bin: convar, primvar,
// alpha_x, alpha_y, then t, the step count and every step's dt.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#ifdef HOS_DRIVER_WITH_REFERENCE
#include "2Dproblem.h"
#else
#include "hos_ref_api.h"
#endif

int main(int argc, char** argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: driver2d config.txt state_in.bin state_out.bin\n");
        return 2;
    }
    std::map<std::string, std::vector<std::string>> cfg;
    {
        std::ifstream in(argv[1]);
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream ls(line);
            std::string key, tok;
            ls >> key;
            if (key.empty()) continue;
            while (ls >> tok) cfg[key].push_back(tok);
        }
    }
    auto num = [&](const char* k, int i = 0) { return std::stod(cfg.at(k).at(i)); };

    Block2d block;
    block.uniform = true;
    block.nodex = (int)num("nodex");
    block.nodey = (int)num("nodey");
    block.ghost = (int)num("ghost");
    block.CFL = num("cfl");
    Fluid2d* bcvalue = new Fluid2d[4];
    K = (int)num("K");
    Gamma = num("gamma");

    std::map<std::string, BoundaryCondition2d> low = {
        {"free", free_boundary_left}, {"periodic", periodic_boundary_left}, {"reflect", reflection_boundary_left},
        {"inflow", inflow_boundary_left}, {"noslip", noslip_adiabatic_boundary_left}};
    std::map<std::string, BoundaryCondition2d> high = {
        {"free", free_boundary_right}, {"periodic", periodic_boundary_right}, {"reflect", reflection_boundary_right},
        {"inflow", inflow_boundary_right}, {"noslip", noslip_adiabatic_boundary_right}};
    std::map<std::string, BoundaryCondition2d> down = {
        {"free", free_boundary_down}, {"periodic", periodic_boundary_down}, {"reflect", reflection_boundary_down},
        {"noslip", noslip_adiabatic_boundary_down}};
    std::map<std::string, BoundaryCondition2d> up = {
        {"free", free_boundary_up}, {"periodic", periodic_boundary_up}, {"reflect", reflection_boundary_up},
        {"inflow", inflow_boundary_up}, {"noslip", noslip_adiabatic_boundary_up}};
    const bool source = cfg.count("source") && num("source") != 0;   // the RT_instability loop
    // (its own RT_boundary fills every side, whose bottom inflow has no side function)
    BoundaryCondition2d leftboundary = source ? nullptr : low.at(cfg.at("bc")[0]);
    BoundaryCondition2d rightboundary = source ? nullptr : high.at(cfg.at("bc")[1]);
    BoundaryCondition2d downboundary = source ? nullptr : down.at(cfg.at("bc")[2]);
    BoundaryCondition2d upboundary = source ? nullptr : up.at(cfg.at("bc")[3]);
    if (cfg.count("bcprim"))
        for (size_t k = 0; k + 5 <= cfg["bcprim"].size(); k += 5) {
            const int side = (int)num("bcprim", (int)k);
            for (int v = 0; v < 4; ++v) bcvalue[side].primvar[v] = num("bcprim", (int)k + 1 + v);
        }

    const int order = (int)num("order");
    gausspoint = order == 5 ? 2 : order == 7 ? 3 : 4;
    SetGuassPoint();
    reconstruction_variable = num("characteristic") != 0 ? characteristic : conservative;
    const std::string wt = cfg.count("wenotype") ? cfg.at("wenotype").at(0) : "z";
    wenotype = wt == "js" ? wenojs : wt == "linear" ? linear : wenoz;
    Reconstruction_within_Cell_2D_normal normal_df =
        order == 5 ? WENO5_AO_with_df_normal : order == 7 ? WENO7_AO_with_df_normal : WENO9_AO_with_df_normal;
    Reconstruction_within_Cell_2D_tangent tangent_df =
        order == 5 ? WENO5_AO_with_df_tangent : order == 7 ? WENO7_AO_with_df_tangent : WENO9_AO_with_df_tangent;
    cellreconstruction_2D_normal = normal_df;
    cellreconstruction_2D_tangent = tangent_df;
    g0reconstruction_2D_normal = Center_do_nothing_normal;
    g0reconstruction_2D_tangent = Center_all_collision_multi;
    is_reduce_order_warning = false;
    is_using_df_factor = !(cfg.count("df") && num("df") == 0);
    if (!is_using_df_factor) {
        cellreconstruction_2D_normal = WENO5_AO_normal;
        cellreconstruction_2D_tangent = WENO5_AO_tangent;
    }
    gks2dsolver = gks2nd_2d;
    tau_type = cfg.count("tau_type") && num("tau_type") == 1 ? NS : Euler;
    if (cfg.count("mu")) Mu = num("mu");
    if (cfg.count("nu")) Nu = num("nu");
    if (cfg.count("prandtl_fix")) is_Prandtl_fix = num("prandtl_fix") != 0;
    if (cfg.count("pr")) Pr = num("pr");
    c1_euler = num("c1");
    c2_euler = num("c2");
    flux_function_2d = GKS2D;
    timecoe_list_2d = S2O4_2D;
    Initial_stages(block);

    block.nx = block.nodex + 2 * block.ghost;
    block.ny = block.nodey + 2 * block.ghost;
    Fluid2d* fluids = Setfluid(block);
    Interface2d* xinterfaces = Setinterface_array(block);
    Interface2d* yinterfaces = Setinterface_array(block);
    Flux2d_gauss** xfluxes = Setflux_gauss_array(block);
    Flux2d_gauss** yfluxes = Setflux_gauss_array(block);
    block.left = num("left");
    block.right = num("right");
    block.down = num("down");
    block.up = num("up");
    block.dx = (block.right - block.left) / block.nodex;
    block.dy = (block.up - block.down) / block.nodey;
    block.overdx = 1 / block.dx;
    block.overdy = 1 / block.dy;
    SetUniformMesh(block, fluids, xinterfaces, yinterfaces, xfluxes, yfluxes);

    const size_t ncell = (size_t)block.nx * block.ny;
    {
        std::vector<double> buf(8 * ncell);
        std::ifstream in(argv[2], std::ios::binary);
        in.read(reinterpret_cast<char*>(buf.data()), (std::streamsize)(buf.size() * sizeof(double)));
        if (!in) {
            std::fprintf(stderr, "short state file\n");
            return 2;
        }
        for (size_t k = 0; k < ncell; ++k)
            for (int v = 0; v < 4; ++v) {
                fluids[k].convar[v] = buf[4 * k + v];
                fluids[k].primvar[v] = buf[4 * ncell + 4 * k + v];
            }
    }
#ifndef HOS_DRIVER_WITH_REFERENCE
    hos_ref_set_precision((int)num("precision"));
    hos_ref_set_mirror((int)num("mirror"));
    hos_ref_set_error_mode(HOS_REF_THROW);
#endif

    const double tstop = num("tstop");
    const int steps = (int)num("steps");
    const int fo_steps = cfg.count("first_order_steps") ? (int)num("first_order_steps") : 0;
    std::vector<double> dts;
    block.t = 0;
    block.step = 0;
#ifndef HOS_DRIVER_WITH_REFERENCE
    try {
#endif
        while (block.t < tstop && block.step < steps) {
            CopyFluid_new_to_old(fluids, block);
            block.dt = Get_CFL(block, fluids, tstop);
            dts.push_back(block.dt);
            if (is_using_df_factor) {
                if (block.step < fo_steps) {
                    cellreconstruction_2D_normal = First_order_normal;
                    cellreconstruction_2D_tangent = First_order_tangent;
                } else {
                    cellreconstruction_2D_normal = normal_df;
                    cellreconstruction_2D_tangent = tangent_df;
                }
            }
            for (int i = 0; i < block.stages; i++) {
                if (source) {
                    RT_boundary(fluids, block);
                } else {
                    leftboundary(fluids, block, bcvalue[0]);
                    rightboundary(fluids, block, bcvalue[1]);
                    downboundary(fluids, block, bcvalue[2]);
                    upboundary(fluids, block, bcvalue[3]);
                }
                Convar_to_Primvar(fluids, block);
                Reconstruction_within_cell(xinterfaces, yinterfaces, fluids, block);
                Reconstruction_forg0(xinterfaces, yinterfaces, fluids, block);
                Calculate_flux(xfluxes, yfluxes, xinterfaces, yinterfaces, block, i);
                if (source) Update_with_source(fluids, xfluxes, yfluxes, block, i);
                else Update(fluids, xfluxes, yfluxes, block, i);
                if (is_using_df_factor) Update_alpha(xinterfaces, yinterfaces, fluids, block);
            }
            block.step++;
            block.t = block.t + block.dt;
        }
#ifndef HOS_DRIVER_WITH_REFERENCE
    } catch (const hos_ref_error& e) {
        std::fprintf(stderr, "hos_ref_error %d: %s\n", e.code, e.what());
        return 3;
    }
    if (!(int)num("mirror")) hos_ref_download2d(fluids, block);
#endif

    std::vector<double> out;
    out.reserve(10 * ncell + 2 + dts.size());
    for (size_t k = 0; k < ncell; ++k)
        for (int v = 0; v < 4; ++v) out.push_back(fluids[k].convar[v]);
    for (size_t k = 0; k < ncell; ++k)
        for (int v = 0; v < 4; ++v) out.push_back(fluids[k].primvar[v]);
    for (size_t k = 0; k < ncell; ++k) out.push_back(fluids[k].alpha_x);
    for (size_t k = 0; k < ncell; ++k) out.push_back(fluids[k].alpha_y);
    out.push_back(block.t);
    out.push_back(block.step);
    out.insert(out.end(), dts.begin(), dts.end());
    std::ofstream o(argv[3], std::ios::binary);
    o.write(reinterpret_cast<const char*>(out.data()), (std::streamsize)(out.size() * sizeof(double)));
    return o ? 0 : 2;
}
