// Driver for the reference FDTD solver (fdtd/fdtd_simulation.cpp), compiled
// against the unmodified reference source by oracle/build_ref.sh.  Oracle test
// infrastructure only: it reads a case description on stdin, runs the
// reference class, and writes its receiver traces and final fields in binary.
//
// stdin:  nx ny nz  h dt eps mu  time_frequency nsteps
//         nsrc   { comp i j k } * nsrc          comp 0/1/2 = setSource_x/y/z
//         nobs   { n0 {i j k}*n0  n1 {...}  n2 {...} } * nobs
// output: int32 nobs, nsamp; double traces[nobs][nsamp][3];
//         then Ex Ey Ez Hx Hy Hz in the reference's padded layout.
#include <array>
#include <vector>
#include <string>
#include <functional>
#include <memory>
#include <cstdio>
#include <iostream>
#define private public
#include "fdtd_simulation.hpp"
#undef private

static void put(FILE *f, const std::vector<double> &v) { fwrite(v.data(), sizeof(double), v.size(), f); }

int main(int argc, char **argv)
{
    if (argc != 2) { std::fprintf(stderr, "usage: fdtd_ref out.bin < case\n"); return 2; }
    int nx, ny, nz, tf, nsteps, nsrc, nobs;
    double h, dt, eps, mu;
    std::cin >> nx >> ny >> nz >> h >> dt >> eps >> mu >> tf >> nsteps >> nsrc;
    FemSimulation sim({nx, ny, nz}, h, dt, eps, mu, tf);
    for (int s = 0; s < nsrc; ++s) {
        int c, i, j, k; std::cin >> c >> i >> j >> k;
        if (c == 0) sim.setSource_x({i, j, k});
        else if (c == 1) sim.setSource_y({i, j, k});
        else sim.setSource_z({i, j, k});
    }
    std::cin >> nobs;
    for (int o = 0; o < nobs; ++o) {
        std::array<std::vector<std::array<int, 3>>, 3> pts;
        for (int c = 0; c < 3; ++c) {
            int n; std::cin >> n;
            for (int q = 0; q < n; ++q) { int i, j, k; std::cin >> i >> j >> k; pts[c].push_back({i, j, k}); }
        }
        sim.setObservationPoint(pts);
    }
    sim.run(nsteps);
    FILE *f = std::fopen(argv[1], "wb");
    if (!f) return 1;
    int hdr[2] = {(int)sim.saved_electric_field_.size(),
                  sim.saved_electric_field_.empty() ? 0 : (int)sim.saved_electric_field_[0].size()};
    fwrite(hdr, sizeof(int), 2, f);
    for (auto &tr : sim.saved_electric_field_)
        for (auto &s : tr) fwrite(s.data(), sizeof(double), 3, f);
    put(f, sim.electric_field_x_); put(f, sim.electric_field_y_); put(f, sim.electric_field_z_);
    put(f, sim.magnetic_field_x_); put(f, sim.magnetic_field_y_); put(f, sim.magnetic_field_z_);
    std::fclose(f);
    return 0;
}
