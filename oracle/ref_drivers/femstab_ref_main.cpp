// Driver for the reference stabilised hexahedral solver (fem/fem_simulation.cpp),
// compiled against the unmodified source by oracle/build_ref.sh.  Oracle test
// infrastructure only.
//
// stdin:  gx gy gz  h dt eps mu  time_frequency  stabilization use_ofem  nsteps
//         nsrc   { comp i j k } * nsrc          setSource_x/_y/_z
//         ndip   { i j k } * ndip               setSourceDipole_x
//         nobs   { n0 {i j k}*n0  n1 {...}  n2 {...} } * nobs
// output: int32 nobs, nsamp; double traces[nobs][nsamp][3];
//         then E_x E_y E_z (3 levels each); then the 12 x 12 element matrix.
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
    if (argc != 2) { std::fprintf(stderr, "usage: femstab_ref out.bin < case\n"); return 2; }
    int gx, gy, gz, tf, ofem, nsteps, nsrc, ndip, nobs;
    double h, dt, eps, mu, sf;
    std::cin >> gx >> gy >> gz >> h >> dt >> eps >> mu >> tf >> sf >> ofem >> nsteps >> nsrc;
    FemSimulation sim({gx, gy, gz}, h, dt, eps, mu, tf, sf, ofem);
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
    for (auto &row : sim.element_stiffness_matrix_) fwrite(row.data(), sizeof(double), 12, f);
    std::fclose(f);
    return 0;
}
