// driver1d.cpp -- a 1D problem driver written against the reference's own function-level API,
// following the loop of SodTubeProblem (src/1Dproblem.cpp:3-148) without its console prompts.
// Built against libhos_ref.so (the GPU path) and, with -DHOS_DRIVER_WITH_REFERENCE, against
// the reference's own sources.
//
//   driver1d <config.txt> <state_in.bin> <state_out.bin>
//
// config.txt: "key value..." lines (nodex ghost order characteristic df K gamma c1 c2 cfl left
// right bc (2 names) steps tstop precision mirror); df is "switch" (WENO5_AO at step 0, then
// WENO5_AO_with_DF, as the Sod driver), "always" or "never".
// state_in.bin: convar [nx][3].  state_out.bin: convar, alpha, then t, step count, every dt.
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#ifdef HOS_DRIVER_WITH_REFERENCE
#include "1Dproblem.h"
#else
#include "hos_ref_api.h"
#endif

int main(int argc, char** argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: driver1d config.txt state_in.bin state_out.bin\n");
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

    Block1d block;
    block.nodex = (int)num("nodex");
    block.ghost = (int)num("ghost");
    block.CFL = num("cfl");
    Fluid1d* bcvalue = new Fluid1d[2];
    K = (int)num("K");
    Gamma = num("gamma");
    R_gas = 1.0;
    gks1dsolver = gks2nd;
    tau_type = Euler;
    c1_euler = num("c1");
    c2_euler = num("c2");
    std::map<std::string, BoundaryCondition> low = {
        {"free", free_boundary_left}, {"reflect", reflection_boundary_left}, {"periodic", periodic_boundary_left}};
    std::map<std::string, BoundaryCondition> high = {
        {"free", free_boundary_right}, {"reflect", reflection_boundary_right}, {"periodic", periodic_boundary_right}};
    BoundaryCondition leftboundary = low.at(cfg.at("bc")[0]);
    BoundaryCondition rightboundary = high.at(cfg.at("bc")[1]);

    const int order = (int)num("order");
    const std::string df = cfg.at("df")[0];
    // WENO5_AO is overloaded in the reference (1D and 2D): select the 1D slot type
    const Reconstruction_within_Cell plain = static_cast<Reconstruction_within_Cell>(WENO5_AO);
    const Reconstruction_within_Cell with_df =
        order == 5 ? WENO5_AO_with_DF : order == 7 ? WENO7_AO_with_DF : WENO9_AO_with_DF;
    cellreconstruction = df == "always" ? with_df : plain;
    is_using_df_factor = df != "never";
    wenotype = wenoz;
    reconstruction_variable = num("characteristic") != 0 ? characteristic : conservative;
    g0reconstruction = Center_collision;
    is_reduce_order_warning = false;
    flux_function = GKS;
    timecoe_list = S2O4;
    Initial_stages(block);

    block.nx = block.nodex + 2 * block.ghost;
    block.nodex_begin = block.ghost;
    block.nodex_end = block.nodex + block.ghost - 1;
    Fluid1d* fluids = new Fluid1d[block.nx];
    Interface1d* interfaces = new Interface1d[block.nx + 1];
    Flux1d** fluxes = Setflux_array(block);
    block.left = num("left");
    block.right = num("right");
    block.dx = (block.right - block.left) / block.nodex;
    SetUniformMesh(block, fluids, interfaces, fluxes);
    {
        std::vector<double> buf(3 * (size_t)block.nx);
        std::ifstream in(argv[2], std::ios::binary);
        in.read(reinterpret_cast<char*>(buf.data()), (std::streamsize)(buf.size() * sizeof(double)));
        if (!in) {
            std::fprintf(stderr, "short state file\n");
            return 2;
        }
        for (int i = 0; i < block.nx; ++i)
            for (int v = 0; v < 3; ++v) fluids[i].convar[v] = buf[3 * i + v];
    }
#ifndef HOS_DRIVER_WITH_REFERENCE
    hos_ref_set_precision((int)num("precision"));
    hos_ref_set_mirror((int)num("mirror"));
    hos_ref_set_error_mode(HOS_REF_THROW);
#endif
    const double tstop = num("tstop");
    const int steps = (int)num("steps");
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
            if (block.step > 0 && is_using_df_factor) cellreconstruction = with_df;
            for (int i = 0; i < block.stages; i++) {
                leftboundary(fluids, block, bcvalue[0]);
                rightboundary(fluids, block, bcvalue[1]);
                Reconstruction_within_cell(interfaces, fluids, block);
                Reconstruction_forg0(interfaces, fluids, block);
                Calculate_flux(fluxes, interfaces, block, i);
                Update(fluids, fluxes, block, i);
                if (is_using_df_factor) Update_alpha(interfaces, fluids, block);
            }
            block.step++;
            block.t = block.t + block.dt;
        }
#ifndef HOS_DRIVER_WITH_REFERENCE
    } catch (const hos_ref_error& e) {
        std::fprintf(stderr, "hos_ref_error %d: %s\n", e.code, e.what());
        return 3;
    }
    if (!(int)num("mirror")) hos_ref_download1d(fluids, block);
#endif
    std::vector<double> out;
    for (int i = 0; i < block.nx; ++i)
        for (int v = 0; v < 3; ++v) out.push_back(fluids[i].convar[v]);
    for (int i = 0; i < block.nx; ++i) out.push_back(fluids[i].alpha);
    out.push_back(block.t);
    out.push_back(block.step);
    out.insert(out.end(), dts.begin(), dts.end());
    std::ofstream o(argv[3], std::ios::binary);
    o.write(reinterpret_cast<const char*>(out.data()), (std::streamsize)(out.size() * sizeof(double)));
    return o ? 0 : 2;
}
