// Order-1 hexahedral edge grid shared by the fem_abm and fem/ solvers
// (fem_abm/fem_simulation.cpp:66-141, fem/fem_simulation.cpp:61-123): the
// three edge families in one concatenated array (x-edges gx(gy+1)(gz+1),
// then y-edges, then z-edges, first coordinate fastest), the cyclic local
// order of a cell's edges, the PEC rule for tangential E, and the
// sequential source and receiver kernels that keep the reference's
// statement order.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <vector>

namespace ems {
namespace {

__device__ __forceinline__ double ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sb(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ml(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float ad(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sb(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float ml(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float dv(float a, float b) { return __fdiv_rn(a, b); }

struct HexGeom {
    int gx, gy, gz;
    size_t n[3];
};

inline HexGeom hex_geom(int gx, int gy, int gz)
{
    HexGeom g{gx, gy, gz, {}};
    g.n[0] = (size_t)gx * (gy + 1) * (gz + 1);
    g.n[1] = (size_t)(gx + 1) * gy * (gz + 1);
    g.n[2] = (size_t)(gx + 1) * (gy + 1) * gz;
    return g;
}

__host__ __device__ __forceinline__ void hex_coords(const HexGeom &g, int c, size_t t, int &i, int &j, int &k)
{
    int nxc = c == 0 ? g.gx : g.gx + 1;
    int nyc = c == 1 ? g.gy : g.gy + 1;
    i = (int)(t % nxc);
    size_t r = t / nxc;
    j = (int)(r % nyc);
    k = (int)(r / nyc);
}

// edge index (within its family) of local edge q of component c in cell
// (i,j,k), cyclic order: x (i, j+q0, k+q1), y (i+q1, j, k+q0), z (i+q0,
// j+q1, k), q = q0 + 2 q1
__host__ __device__ __forceinline__ size_t hex_edge(const HexGeom &g, int c, int i, int j, int k, int q)
{
    int a0 = q & 1, a1 = q >> 1;
    const int gx = g.gx, gy = g.gy;
    if (c == 0) return (size_t)i + (size_t)(j + a0) * gx + (size_t)(k + a1) * gx * (gy + 1);
    if (c == 1) return (size_t)(i + a1) + (size_t)j * (gx + 1) + (size_t)(k + a0) * (gx + 1) * gy;
    return (size_t)(i + a0) + (size_t)(j + a1) * (gx + 1) + (size_t)k * (gx + 1) * (gy + 1);
}

// tangential E on a face of the box
__host__ __device__ __forceinline__ bool hex_e_pec(const HexGeom &g, int c, int i, int j, int k)
{
    if (c == 0) return j == 0 || j == g.gy || k == 0 || k == g.gz;
    if (c == 1) return i == 0 || i == g.gx || k == 0 || k == g.gz;
    return i == 0 || i == g.gx || j == 0 || j == g.gy;
}

// Point sources and dipole weights in the reference's statement order.
// op: 0 = subtract, 1 = add.  Entries on PEC-zeroed DOFs are skipped when
// `bc` is set (the reference zeroes them right after).
template <class T>
__global__ void hex_source_kernel(HexGeom g, T *E2, int n, const long long *idx, const double *val, const int *op, int bc)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int s = 0; s < n; ++s) {
        size_t q = (size_t)idx[s];
        if (bc) {
            int c = q < g.n[0] ? 0 : (q < g.n[0] + g.n[1] ? 1 : 2);
            size_t t = q - (c == 0 ? 0 : (c == 1 ? g.n[0] : g.n[0] + g.n[1]));
            int i, j, k;
            hex_coords(g, c, t, i, j, k);
            if (hex_e_pec(g, c, i, j, k)) continue;
        }
        T v = (T)val[s];
        E2[q] = op[s] ? ad(E2[q], v) : sb(E2[q], v);
    }
}

// Receivers: sums over listed edges of E2, divided by the count
// (fem_abm/fem_simulation.cpp:972-1013, fem/fem_simulation.cpp:856-903).
template <class T>
__global__ void hex_sample_kernel(int nobs, const int *cnt, const int *start, const long long *idx, const T *E2, double *tr,
                                  int nsamp, int s)
{
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nobs) return;
    double *out = tr + ((size_t)o * nsamp + s) * 3;
    int q = start[o];
    for (int c = 0; c < 3; ++c) {
        int n = cnt[3 * o + c];
        double acc = out[c];
        for (int r = 0; r < n; ++r, ++q) acc = __dadd_rn(acc, (double)E2[idx[q]]);
        out[c] = acc / (double)n;
    }
}

// Flat index (families concatenated) of edge (i,j,k) of component c.
inline long long hex_flat(const HexGeom &g, int c, int i, int j, int k)
{
    const int gx = g.gx, gy = g.gy;
    size_t t = c == 0 ? (size_t)i + (size_t)j * gx + (size_t)k * gx * (gy + 1)
             : c == 1 ? (size_t)i + (size_t)j * (gx + 1) + (size_t)k * (gx + 1) * gy
                      : (size_t)i + (size_t)j * (gx + 1) + (size_t)k * (gx + 1) * (gy + 1);
    return (long long)((c == 0 ? 0 : (c == 1 ? g.n[0] : g.n[0] + g.n[1])) + t);
}

// The x-directed Hertz dipole over the cells (i, j..j+1, k..k+1) as the
// reference states it (fem_abm/fem_simulation.cpp:407-481,
// fem/fem_simulation.cpp:636-705): nine x-edges with weights 1/8, 3/4, 9/2,
// and the stabilisation terms sf/2 on eight y-edges and eight z-edges, in
// statement order; appended as (edge, weight, +1 add / 0 subtract).
inline void hex_dipole_terms(const HexGeom &g, const std::array<int, 3> &p, double sf, std::vector<long long> &idx,
                             std::vector<double> &wt, std::vector<int> &op)
{
    int i = p[0], j = p[1], k = p[2];
    auto X = [&](int ci, int cj, int ck, int q) { return hex_flat(g, 0, ci, cj + (q & 1), ck + (q >> 1)); };
    auto Y = [&](int ci, int cj, int ck, int q) { return hex_flat(g, 1, ci + (q >> 1), cj, ck + (q & 1)); };
    auto Z = [&](int ci, int cj, int ck, int q) { return hex_flat(g, 2, ci + (q & 1), cj + (q >> 1), ck); };
    // cells c0 = (i,j,k), c1 = (i,j+1,k), c2 = (i,j,k+1), c3 = (i,j+1,k+1)
    const int C[4][3] = {{i, j, k}, {i, j + 1, k}, {i, j, k + 1}, {i, j + 1, k + 1}};
    struct Term { int comp, cell, q; double w; int add; };
    const double s2 = sf / 2.0;
    const Term terms[] = {
        {0, 0, 0, 1.0 / 8.0, 1}, {0, 0, 1, 3.0 / 4.0, 1}, {0, 0, 2, 3.0 / 4.0, 1}, {0, 0, 3, 9.0 / 2.0, 1},
        {0, 1, 1, 1.0 / 8.0, 1}, {0, 1, 3, 3.0 / 4.0, 1}, {0, 2, 2, 1.0 / 8.0, 1}, {0, 2, 3, 3.0 / 4.0, 1},
        {0, 3, 3, 1.0 / 8.0, 1},
        {1, 0, 0, s2, 1}, {1, 0, 2, s2, 1}, {1, 1, 0, s2, 1}, {1, 1, 2, s2, 1},
        {1, 2, 1, s2, 0}, {1, 2, 3, s2, 0}, {1, 3, 1, s2, 0}, {1, 3, 3, s2, 0},
        {2, 0, 0, s2, 0}, {2, 0, 1, s2, 0}, {2, 1, 2, s2, 1}, {2, 1, 3, s2, 1},
        {2, 2, 0, s2, 0}, {2, 2, 1, s2, 0}, {2, 3, 2, s2, 1}, {2, 3, 3, s2, 1}};
    for (const Term &t : terms) {
        const int *cc = C[t.cell];
        long long e = t.comp == 0 ? X(cc[0], cc[1], cc[2], t.q) : t.comp == 1 ? Y(cc[0], cc[1], cc[2], t.q) : Z(cc[0], cc[1], cc[2], t.q);
        idx.push_back(e);
        wt.push_back(t.w);
        op.push_back(t.add);
    }
}

}  // namespace
}  // namespace ems
