// hos_ref_output.cpp -- the reference's ASCII writers (src/output.cpp:3-84): the same file
// names, row order and stream formatting, so the reference's plotting and diff scripts read
// GPU results unchanged.  With mirroring on, the Fluid arrays hold the device state after
// every step; otherwise call hos_ref_download1d/2d first.
#include <cmath>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>

#include "hos_ref_api.h"

void output1d(Fluid1d* fluids, Block1d block) {
    std::ofstream out("../data/R.txt");
    for (int i = block.ghost; i < block.nodex + block.ghost; ++i) out << fluids[i].convar[0] << std::endl;
}

// density of the interior cells, x fastest then y, one value per line (file R-<step>.txt)
void output2d(Fluid2d* fluids, Block2d block) {
    std::stringstream name;
    name << "../data/R-" << block.step << ".txt";
    std::string path;
    name >> path;
    std::ofstream out(path, std::ios::trunc);
    for (int j = block.ghost; j < block.ghost + block.nodey; ++j)
        for (int i = block.ghost; i < block.ghost + block.nodex; ++i)
            out << fluids[(size_t)i * block.ny + j].convar[0] << std::endl;
}

// L1 / L2 / Linf errors per mesh with the observed orders between successive meshes, as a
// LaTeX table body (error.txt)
void output_error_form(double CFL, double dt_ratio, int mesh_set, int* mesh_number, double** error) {
    std::cout << "Accuracy-residual-file-output" << std::endl;
    std::ofstream out("../data/error.txt");
    out << "the CFL number is " << CFL << std::endl;
    out << "the dt ratio over dx is " << dt_ratio << std::endl;
    for (int i = 0; i < mesh_set; ++i) {
        if (i == 0) {
            out << "1/" << mesh_number[i] << std::scientific << std::setprecision(6) << " & " << error[i][0] << " & ~"
                << " & " << error[i][1] << " & ~"
                << " & " << error[i][2] << " & ~"
                << " \\\\ " << std::endl;
            continue;
        }
        out << "1/" << mesh_number[i];
        for (int m = 0; m < 3; ++m) {
            const double order = std::log(error[i - 1][m] / error[i][m]) / std::log(2);
            out << " & " << std::scientific << std::setprecision(6) << error[i][m];
            out << " & " << std::fixed << std::setprecision(2) << order;
        }
        out << " \\\\ " << std::endl;
    }
}
