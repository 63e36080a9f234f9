// outputs.cpp -- writes the reference's ASCII outputs (output1d, output2d, output_error_form)
// for fixed synthetic data; built against the reference (-DHOS_DRIVER_WITH_REFERENCE) and
// against libhos_ref.so so the tests can compare the files byte for byte.  Run it in a
// directory whose parent holds data/.
#include <cmath>

#ifdef HOS_DRIVER_WITH_REFERENCE
#include "2Dproblem.h"
#include "output.h"
#else
#include "hos_ref_api.h"
#endif

int main() {
    Block2d b2;
    b2.nodex = 7;
    b2.nodey = 5;
    b2.ghost = 3;
    b2.nx = b2.nodex + 2 * b2.ghost;
    b2.ny = b2.nodey + 2 * b2.ghost;
    b2.step = 42;
    Fluid2d* f2 = new Fluid2d[b2.nx * b2.ny];
    for (int k = 0; k < b2.nx * b2.ny; ++k) f2[k].convar[0] = 1.0 + 0.37 * std::sin(0.7 * k) * std::pow(10.0, (k % 9) - 4);
    output2d(f2, b2);
    Block1d b1;
    b1.nodex = 11;
    b1.ghost = 2;
    b1.nx = b1.nodex + 2 * b1.ghost;
    Fluid1d* f1 = new Fluid1d[b1.nx];
    for (int k = 0; k < b1.nx; ++k) f1[k].convar[0] = 0.125 + k / 3.0;
    output1d(f1, b1);
    int meshes[3] = {10, 20, 40};
    double e0[3] = {1.2e-3, 4.5e-4, 3.3e-6}, e1[3] = {3.8e-5, 1.1e-6, 9.9e-8}, e2[3] = {1.2e-6, 4.0e-8, 1.3e-9};
    double* err[3] = {e0, e1, e2};
    output_error_form(0.5, 0.25, 3, meshes, err);
    return 0;
}
