// Driver for the reference Adams-Bashforth-Moulton solver
// (fem_abm/fem_simulation.cpp), compiled against the unmodified source by
// oracle/build_ref.sh.  Oracle test infrastructure only.
//
// stdin:  gx gy gz  h dt eps mu  time_frequency nsteps
//         nsrc   { comp i j k } * nsrc          setSource_x/_y/_z
//         ndip   { i j k } * ndip               setSourceDipole_x
//         nobs   { n0 {i j k}*n0  n1 {...}  n2 {...} } * nobs
// output: int32 nobs, nsamp; double traces[nobs][nsamp][3];
//         then E_x E_y E_z H_x H_y H_z (4 levels each).
#include <array>
#include <vector>
#include <string>
#include <functional>
#include <memory>
#include <cstdio>
#include <iostream>
#define private public
#include "fem_simulation.hpp"
#undef private

static void put(FILE *f, const std::vector<double> &v) { fwrite(v.data(), sizeof(double), v.size(), f); }

int main(int argc, char **argv)
{
    if (argc != 2) { std::fprintf(stderr, "usage: abm_ref out.bin < case\n"); return 2; }
    int gx, gy, gz, tf, nsteps, nsrc, ndip, nobs;
    double h, dt, eps, mu;
    std::cin >> gx >> gy >> gz >> h >> dt >> eps >> mu >> tf >> nsteps >> nsrc;
    FemSimulation sim({gx, gy, gz}, h, dt, eps, mu, tf);
    for (int s = 0; s < nsrc; ++s) {
        int c, i, j, k; std::cin >> c >> i >> j >> k;
        if (c == 0) sim.setSource_x({i, j, k});
        else if (c == 1) sim.setSource_y({i, j, k});
        else sim.setSource_z({i, j, k});
    }
    std::cin >> ndip;
    for (int s = 0; s < ndip; ++s) { int i, j, k; std::cin >> i >> j >> k; sim.setSourceDipole_x({i, j, k}); }
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
