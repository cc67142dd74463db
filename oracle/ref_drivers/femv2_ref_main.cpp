// Driver for the reference hexahedral FEM solvers of the fem_v2 family
// (fem_v2 leapfrog, symplectic_2, symplectic_4 — all share one class
// interface), compiled against each variant's unmodified source by
// oracle/build_ref.sh.  Oracle test infrastructure only: one rank, dims
// (1,1,1); it runs the reference class and dumps traces and fields.
//
// argv: out.bin kmat_parent_dir order use_ofem nx ny nz h dt eps mu tf nsteps
//       src_comp si sj sk  oi oj ok
// output: int32 nsamp; double traces[nsamp][4] (t,Ex,Ey,Ez);
//         int32 n_x n_y n_z; double ef_x[n_x] ef_y[n_y] ef_z[n_z] (all levels)
#include <array>
#include <vector>
#include <string>
#include <functional>
#include <memory>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <unistd.h>
#include <mpi.h>
#define private public
#include "fem_simulation.hpp"
#undef private

int main(int argc, char **argv)
{
    if (argc != 21) { std::fprintf(stderr, "usage: see header\n"); return 2; }
    std::string out = argv[1];
    if (out[0] != '/') { char cwd[4096]; if (!getcwd(cwd, sizeof cwd)) return 2; out = std::string(cwd) + "/" + out; }
    if (chdir(argv[2]) != 0) { std::perror("chdir"); return 2; }
    int order = std::atoi(argv[3]), use_ofem = std::atoi(argv[4]);
    std::array<int, 3> grid = {std::atoi(argv[5]), std::atoi(argv[6]), std::atoi(argv[7])};
    double h = std::atof(argv[8]), dt = std::atof(argv[9]), eps = std::atof(argv[10]), mu = std::atof(argv[11]);
    int tf = std::atoi(argv[12]), nsteps = std::atoi(argv[13]);
    int sc = std::atoi(argv[14]);
    std::array<int, 3> src = {std::atoi(argv[15]), std::atoi(argv[16]), std::atoi(argv[17])};
    std::array<int, 3> obs = {std::atoi(argv[18]), std::atoi(argv[19]), std::atoi(argv[20])};
    std::array<int, 3> dims = {1, 1, 1}, coords = {0, 0, 0};
    MPI_Comm c = 0;
    FemSimulation sim(order, grid, h, dt, eps, mu, tf, use_ofem, dims, coords, 0,
                      c, c, c, c, c, c, c, c, c, c, c, c, c, c, c, c, c, c,
                      0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0);
    if (sc == 0) sim.setSource_x(src);
    else if (sc == 1) sim.setSource_y(src);
    else sim.setSource_z(src);
    sim.setObservationPoint(obs);
    sim.run(nsteps);
    FILE *f = std::fopen(out.c_str(), "wb");
    if (!f) return 1;
    int ns = sim.saved_electric_field_.empty() ? 0 : (int)sim.saved_electric_field_[0].size();
    fwrite(&ns, sizeof(int), 1, f);
    if (ns) for (auto &s : sim.saved_electric_field_[0]) fwrite(s.data(), sizeof(double), 4, f);
    int n3[3] = {(int)sim.electric_field_x_.size(), (int)sim.electric_field_y_.size(), (int)sim.electric_field_z_.size()};
    fwrite(n3, sizeof(int), 3, f);
    fwrite(sim.electric_field_x_.data(), sizeof(double), n3[0], f);
    fwrite(sim.electric_field_y_.data(), sizeof(double), n3[1], f);
    fwrite(sim.electric_field_z_.data(), sizeof(double), n3[2], f);
    std::fclose(f);
    return 0;
}
