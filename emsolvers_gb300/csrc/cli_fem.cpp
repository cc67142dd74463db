// ems_fem: command-line driver with the argument list of the reference's
// fem_v2 / symplectic_2 / symplectic_4 programs (fem_v2/main.cpp:51-115):
//
//   ems_fem <scale> <use_ofem> <order> <domain_size_x> <domain_size_y>
//           <domain_size_z> <base_num> <duration> <source_position_x>
//           <source_position_y> <source_position_z> <observation_position_x>
//           <observation_position_y> <observation_position_z> <dim_x> <dim_y> <dim_z>
//
// Same derived quantities as the reference: grid = scale*base_num per axis,
// h = domain_size_x/grid, dt = h/(c sqrt(3))/2, time_frequency = 2*scale,
// steps = floor(duration/dt)+1, source and observation indices rounded from
// the positions, a z-directed point source, and the same output file name.
// The whole domain runs on one GPU, so dim_x/y/z are accepted and ignored.
// EMS_INTEGRATOR = leapfrog (default, fem_v2) | symp2 | symp4 selects the
// time step; EMS_PRECISION = fp64 (default) | fp32; EMS_KMAT_DIR overrides
// the element-matrix directory (default "kmat", as the reference).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>

#include "ems.h"

namespace ems {
// the reference's number format in result file names (libems, common.cpp)
std::string compress_number(double v);
}

int main(int argc, char *argv[])
{
    if (argc != 18) {
        std::cout << "Usage: ems_fem <scale> <use_ofem> <order> <domain_size_x> <domain_size_y> <domain_size_z> "
                     "<base_num> <duration> <source_position_x> <source_position_y> <source_position_z> "
                     "<observation_position_x> <observation_position_y> <observation_position_z> <dim_x> <dim_y> <dim_z>"
                  << std::endl;
        return 1;
    }
    int scale = std::stoi(argv[1]), use_ofem = std::stoi(argv[2]), order = std::stoi(argv[3]);
    double dsx = std::stod(argv[4]), dsy = std::stod(argv[5]), dsz = std::stod(argv[6]);
    int base_num = std::stoi(argv[7]);
    double duration = std::stod(argv[8]);
    double sp[3] = {std::stod(argv[9]), std::stod(argv[10]), std::stod(argv[11])};
    double op[3] = {std::stod(argv[12]), std::stod(argv[13]), std::stod(argv[14])};
    const double permittivity = 1.0 * 8.8541878128e-12, permeability = 1.0 * 1.25663706212e-6;
    const double c = 1.0 / std::sqrt(permittivity * permeability);
    int grid = scale * base_num;
    double h = dsx / grid;
    int src[3], obs[3];
    for (int q = 0; q < 3; ++q) {
        src[q] = (int)std::round(sp[q] / h);
        obs[q] = (int)std::round(op[q] / h);
    }
    double dt = h / (c * std::sqrt(3.0)) / 2.0;
    int tf = scale * 2;
    int nsteps = (int)(std::floor(duration / dt) + 1);

    std::string integ = std::getenv("EMS_INTEGRATOR") ? std::getenv("EMS_INTEGRATOR") : "leapfrog";
    std::string prefix;
    ems_hexfem_params p{};
    if (integ == "symp2") { p.integrator = EMS_SYMP2; prefix = "symplectic2nd"; }
    else if (integ == "symp4") { p.integrator = EMS_SYMP4; prefix = "symplectic4th"; }
    else if (integ == "leapfrog") { p.integrator = EMS_LEAPFROG; prefix = ""; }
    else { std::cerr << "EMS_INTEGRATOR must be leapfrog, symp2 or symp4" << std::endl; return 1; }
    std::string filename = prefix + (use_ofem ? "ofem" : "fem") + std::to_string(order) + "_" + std::to_string(scale) + "_" +
                           ems::compress_number(dsx) + "_" + ems::compress_number(dsy) + "_" + ems::compress_number(dsz) + "_" + ems::compress_number(duration) + "_" +
                           ems::compress_number(sp[0]) + "_" + ems::compress_number(sp[1]) + "_" + ems::compress_number(sp[2]) + "_" + ems::compress_number(op[0]) + "_" +
                           ems::compress_number(op[1]) + "_" + ems::compress_number(op[2]) + ".csv";
    // check_params (fem_v2/fem_simulation.cpp:1355-1388)
    if (dsx <= 0 || dsy <= 0 || dsz <= 0 || grid <= 0 || duration <= 0 || dt <= 0 ||
        std::round(dsx / grid) != std::round(dsy / grid) || std::round(dsx / grid) != std::round(dsz / grid) || c * dt >= h) {
        std::cerr << "Invalid parameters" << std::endl;
        return 1;
    }
    p.order = order;
    p.grid[0] = p.grid[1] = p.grid[2] = grid;
    p.h = h;
    p.dt = dt;
    p.permittivity = permittivity;
    p.permeability = permeability;
    p.time_frequency = tf;
    p.use_ofem = use_ofem;
    const char *prec = std::getenv("EMS_PRECISION");
    p.precision = (prec && std::strcmp(prec, "fp32") == 0) ? EMS_FP32 : EMS_FP64;
    p.kmat_dir = std::getenv("EMS_KMAT_DIR") ? std::getenv("EMS_KMAT_DIR") : "kmat";
    ems_sim *sim = nullptr;
    if (ems_hexfem_create(&p, &sim) != EMS_OK) {
        std::cerr << "error: " << ems_last_error(nullptr) << std::endl;
        return 1;
    }
    int rc = ems_hexfem_set_source(sim, 2, src);
    if (rc == EMS_OK) rc = ems_hexfem_add_observation(sim, obs);
    if (rc == EMS_OK) rc = ems_run(sim, nsteps);
    if (rc == EMS_OK) rc = ems_save_results(sim, filename.c_str());
    if (rc != EMS_OK) {
        std::cerr << "error: " << ems_last_error(sim) << std::endl;
        ems_destroy(sim);
        return 1;
    }
    double ms = 0;
    long long launches = 0;
    ems_last_run_stats(sim, &ms, &launches);
    std::cout << "steps: " << nsteps << " device time: " << ms << " ms; results saved to " << filename << std::endl;
    ems_destroy(sim);
    return 0;
}
