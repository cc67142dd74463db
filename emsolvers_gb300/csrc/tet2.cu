// Second-order (20-DOF) Nedelec tetrahedra on Kuhn-split cubes, one GPU.
//
// The reference's higher-order edge elements are the hexahedral fem_v2
// family (fem_v2/fem_kernels.hpp:6-8,13-86: per element, gather the DOFs,
// contract them with the reference matrix of the order, scatter back); its
// time loops are symplectic_2/fem_simulation.cpp:557-672 (drift, force,
// kick, drift), symplectic_4/fem_simulation.cpp:1347-1350 (triple jump) and
// fem_v2/fem_simulation.cpp:627-654 (three-level leapfrog).  This solver
// runs those loops on the complete second-order Nedelec space of a cube mesh
// split into six Kuhn tetrahedra:
//
//   space        per tetrahedron, with barycentrics l and Whitney functions
//                w_ij: edge (i,j) tail (l_i - 5/8 (l_k + l_l)) w_ij and head
//                (l_j - 5/8 (l_k + l_l)) w_ij, face (i,j,k) l_k w_ij and
//                l_i w_jk (vertices in the global node order).
//   layout       38 planes per node, DOF = plane * nnode + node (node = the
//                entity's lowest vertex): 0..6 edge tails, 7..13 edge heads
//                of the 7 edge directions, 14 + 2 f and 15 + 2 f the two
//                functions of face type f.  Tetrahedra in type-major order
//                (p * ncube + cube) so that a warp reads one type's tables.
//   stiffness    element by element through the curl: the curl of the 20
//                functions is linear, so the element computes its values at
//                the four vertices (dyadic coefficients), the P1 mass of
//                those values and the transposed curl; FP64 for FP64 runs,
//                double-float (compensated FP32) for FP32 runs, the kick
//                summed and applied to P in FP64: the kick of an FP32 run is
//                the one place where rounding accumulates without bound, in
//                the null space of K.
//   mass inverse the drift applies q(M) P, the degree-m Chebyshev polynomial
//                of the mass preconditioned by its 2 x 2 edge and face
//                blocks, on the element bounds of the preconditioned
//                spectrum; one entity pass per iteration: each edge or face
//                forms its two mass rows from the iterate of its (up to six)
//                tetrahedra in a fixed order (no atomics, no per-tetrahedron
//                array), applies the block inverse and the Chebyshev update,
//                and writes the next iterate to the other of two buffers.
//   time loop    one CUDA graph per step, replayed; a device step counter
//                indexes the source table and the receiver samples.
// Units are normalised (cube edge 1, c0 = 1); the API converts.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <type_traits>
#include <utility>
#include <vector>

#include "ems_internal.hpp"

namespace ems {

double tet_wave_value(int kind, double f0, double t);
double tet_stability_constant(int integrator);

namespace {

constexpr int kEnt = 19;       // entity types per node: 7 edge directions, 12 face types
constexpr int kPlanes = 38;    // DOF planes per node
constexpr int kMaxInc = 6;     // tetrahedra around one entity
constexpr int kPerm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
constexpr int kEdge[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
constexpr int kFace[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
constexpr int kDir[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
constexpr double kAdmix = -0.625;
constexpr int kMassIters = 28;

// ------------------------------------------------------- element geometry
struct Kuhn {
    double g[4][3];   // gradients of the barycentrics
    int vert[4][3];   // vertex offsets in the cube
};

Kuhn kuhn(int p)
{
    Kuhn k{};
    const int a = kPerm[p][0], b = kPerm[p][1], c = kPerm[p][2];
    k.g[0][a] = -1; k.g[1][a] = 1; k.g[1][b] = -1; k.g[2][b] = 1; k.g[2][c] = -1; k.g[3][c] = 1;
    k.vert[1][a] = 1; k.vert[2][a] = 1; k.vert[2][b] = 1;
    k.vert[3][0] = k.vert[3][1] = k.vert[3][2] = 1;
    return k;
}

int dir_of(const int d[3])
{
    for (int k = 0; k < 7; ++k)
        if (kDir[k][0] == d[0] && kDir[k][1] == d[1] && kDir[k][2] == d[2]) return k;
    return -1;
}
// face types: ordered pairs (S1, S2) of disjoint non-empty axis sets (bit q =
// axis q) in the order s1 = 1..7, s2 = 1..7
int face_type(int s1, int s2)
{
    int t = 0;
    for (int a = 1; a < 8; ++a)
        for (int b = 1; b < 8; ++b) {
            if (a & b) continue;
            if (a == s1 && b == s2) return t;
            ++t;
        }
    return -1;
}
int face_axes(int f)   // S1 | S2 of face type f
{
    int t = 0;
    for (int a = 1; a < 8; ++a)
        for (int b = 1; b < 8; ++b) {
            if (a & b) continue;
            if (t++ == f) return a | b;
        }
    return 0;
}
int bits(const int d[3]) { return (d[0] ? 1 : 0) | (d[1] ? 2 : 0) | (d[2] ? 4 : 0); }

// Function a of type p as (sum_n co[n] l_n) w_ij.
struct Fun {
    double co[4];
    int i, j;
};
Fun fun(int a)
{
    Fun f{};
    if (a < 12) {
        const int l = a % 6;
        f.i = kEdge[l][0]; f.j = kEdge[l][1];
        for (int k = 0; k < 4; ++k) f.co[k] = (k == f.i || k == f.j) ? 0.0 : kAdmix;
        f.co[a < 6 ? f.i : f.j] = 1.0;
    } else {
        const int *v = kFace[(a - 12) / 2];
        if ((a - 12) % 2 == 0) { f.co[v[2]] = 1.0; f.i = v[0]; f.j = v[1]; }
        else { f.co[v[0]] = 1.0; f.i = v[1]; f.j = v[2]; }
    }
    return f;
}

// plane and lowest local vertex of local DOF a of type p
void local_dof(int p, int a, int &plane, int &low)
{
    const Kuhn k = kuhn(p);
    if (a < 12) {
        const int l = a % 6, i = kEdge[l][0], j = kEdge[l][1];
        const int d[3] = {k.vert[j][0] - k.vert[i][0], k.vert[j][1] - k.vert[i][1], k.vert[j][2] - k.vert[i][2]};
        plane = dir_of(d) + (a < 6 ? 0 : 7);
        low = i;
    } else {
        const int *v = kFace[(a - 12) / 2];
        int d1[3], d2[3];
        for (int q = 0; q < 3; ++q) { d1[q] = k.vert[v[1]][q] - k.vert[v[0]][q]; d2[q] = k.vert[v[2]][q] - k.vert[v[1]][q]; }
        plane = 14 + 2 * face_type(bits(d1), bits(d2)) + (a - 12) % 2;
        low = v[0];
    }
}

void cross(const double *x, const double *y, double *r)
{
    r[0] = x[1] * y[2] - x[2] * y[1];
    r[1] = x[2] * y[0] - x[0] * y[2];
    r[2] = x[0] * y[1] - x[1] * y[0];
}

// The 20 function values at barycentric point lam.
void values(int p, const double lam[4], double val[20][3])
{
    const Kuhn k = kuhn(p);
    for (int a = 0; a < 20; ++a) {
        const Fun f = fun(a);
        double pre = 0.0;
        for (int n = 0; n < 4; ++n) pre += f.co[n] * lam[n];
        for (int q = 0; q < 3; ++q) val[a][q] = pre * (lam[f.i] * k.g[f.j][q] - lam[f.j] * k.g[f.i][q]);
    }
}

// Curl of function a at the four vertices (the curl is linear):
// curl((sum co_n l_n) w_ij) = sum_v l_v C_v with
// C_v = 2 co_v grad l_i x grad l_j + [v = i] G_j - [v = j] G_i,
// G_m = sum_n co_n grad l_n x grad l_m.
void curls(int p, double C[20][12])
{
    const Kuhn k = kuhn(p);
    for (int a = 0; a < 20; ++a) {
        const Fun f = fun(a);
        double gij[3], Gi[3] = {0, 0, 0}, Gj[3] = {0, 0, 0}, t[3];
        cross(k.g[f.i], k.g[f.j], gij);
        for (int n = 0; n < 4; ++n) {
            cross(k.g[n], k.g[f.j], t);
            for (int q = 0; q < 3; ++q) Gj[q] += f.co[n] * t[q];
            cross(k.g[n], k.g[f.i], t);
            for (int q = 0; q < 3; ++q) Gi[q] += f.co[n] * t[q];
        }
        for (int v = 0; v < 4; ++v)
            for (int q = 0; q < 3; ++q)
                C[a][3 * v + q] = 2.0 * f.co[v] * gij[q] + (v == f.i ? Gj[q] : 0.0) - (v == f.j ? Gi[q] : 0.0);
    }
}

// Element mass (eps = 1) by a collapsed-coordinate Gauss-Legendre rule, 4
// points per direction (exact for the degree-4 integrands with the
// collapse Jacobian (1-u)^2 (1-v)); the barycentric integrals of an affine
// image of the unit tetrahedron are those of the unit tetrahedron (|T| = 1/6).
void element_mass(int p, double M[400])
{
    const double s = std::sqrt(6.0 / 5.0);
    const double xi[4] = {-std::sqrt(3.0 / 7.0 + 2.0 / 7.0 * s), -std::sqrt(3.0 / 7.0 - 2.0 / 7.0 * s),
                          std::sqrt(3.0 / 7.0 - 2.0 / 7.0 * s), std::sqrt(3.0 / 7.0 + 2.0 / 7.0 * s)};
    const double wo = (18.0 - std::sqrt(30.0)) / 36.0, wi = (18.0 + std::sqrt(30.0)) / 36.0;
    const double wq[4] = {wo, wi, wi, wo};
    std::fill(M, M + 400, 0.0);
    for (int iu = 0; iu < 4; ++iu)
        for (int iv = 0; iv < 4; ++iv)
            for (int iw = 0; iw < 4; ++iw) {
                const double u = 0.5 * (1 + xi[iu]), v = 0.5 * (1 + xi[iv]), w = 0.5 * (1 + xi[iw]);
                const double x = u, y = v * (1 - u), z = w * (1 - u) * (1 - v);
                const double W = 0.125 * wq[iu] * wq[iv] * wq[iw] * (1 - u) * (1 - u) * (1 - v);
                const double lam[4] = {1 - x - y - z, x, y, z};
                double val[20][3];
                values(p, lam, val);
                for (int a = 0; a < 20; ++a)
                    for (int b = 0; b < 20; ++b)
                        M[20 * a + b] += W * (val[a][0] * val[b][0] + val[a][1] * val[b][1] + val[a][2] * val[b][2]);
            }
}

// Element stiffness (mu = 1) from the vertex curls: int l_v l_w = |T| (1 + d_vw) / 20.
void element_stiffness(int p, double K[400])
{
    double C[20][12];
    curls(p, C);
    for (int a = 0; a < 20; ++a)
        for (int b = 0; b < 20; ++b) {
            double s = 0.0;
            for (int v = 0; v < 4; ++v)
                for (int w = 0; w < 4; ++w) {
                    const double d = C[a][3 * v] * C[b][3 * w] + C[a][3 * v + 1] * C[b][3 * w + 1] + C[a][3 * v + 2] * C[b][3 * w + 2];
                    s += d * (v == w ? 2.0 : 1.0) / 120.0;
                }
            K[20 * a + b] = s;
        }
}

// eigenvalues of a symmetric n x n matrix by cyclic Jacobi rotations
void sym_eigs(int n, std::vector<double> A, std::vector<double> &w)
{
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j) off += A[i * n + j] * A[i * n + j];
        if (off < 1e-30) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[p * n + q];
                if (std::fabs(apq) < 1e-300) continue;
                const double th = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
            }
    }
    w.resize(n);
    for (int i = 0; i < n; ++i) w[i] = A[i * n + i];
    std::sort(w.begin(), w.end());
}

// Bounds of the generalised eigenvalues of (M_T, its 2 x 2 entity blocks)
// over the six types: the spectrum of the block-preconditioned global mass
// lies inside (assembly of element inequalities), whatever eps.
void cheb_bounds(const double Mref[6][400], double &lo, double &hi)
{
    lo = 1e300; hi = 0.0;
    for (int p = 0; p < 6; ++p) {
        const double *M = Mref[p];
        std::vector<double> Li(400, 0.0), T(400), A(400), w;
        for (int e = 0; e < 10; ++e) {
            const int i0 = e < 6 ? e : 12 + 2 * (e - 6), i1 = e < 6 ? e + 6 : 13 + 2 * (e - 6);
            const double l00 = std::sqrt(M[20 * i0 + i0]), l10 = M[20 * i0 + i1] / l00;
            const double l11 = std::sqrt(M[20 * i1 + i1] - l10 * l10);
            Li[20 * i0 + i0] = 1.0 / l00;
            Li[20 * i1 + i1] = 1.0 / l11;
            Li[20 * i1 + i0] = -l10 / (l00 * l11);
        }
        for (int i = 0; i < 20; ++i)
            for (int j = 0; j < 20; ++j) {
                double s = 0.0;
                for (int k = 0; k < 20; ++k) s += Li[20 * i + k] * M[20 * k + j];
                T[20 * i + j] = s;
            }
        for (int i = 0; i < 20; ++i)
            for (int j = 0; j < 20; ++j) {
                double s = 0.0;
                for (int k = 0; k < 20; ++k) s += T[20 * i + k] * Li[20 * j + k];
                A[20 * i + j] = s;
            }
        sym_eigs(20, A, w);
        lo = std::min(lo, w.front());
        hi = std::max(hi, w.back());
    }
}

// Reference data of the element, computed once per process.
struct Ref {
    double M[6][400], K[6][400], C[6][20][12];
    int plane[6][20], low[6][20];
    double lo, hi;
    // per entity type: incidences packed p | cube-offset bits << 3 | la << 6 | lb << 11
    int ninc[kEnt], inc[kEnt][kMaxInc];
    int axes[kEnt];   // axes the entity spans (bit q)
    Ref()
    {
        for (int p = 0; p < 6; ++p) {
            element_mass(p, M[p]);
            element_stiffness(p, K[p]);
            curls(p, C[p]);
            for (int a = 0; a < 20; ++a) local_dof(p, a, plane[p][a], low[p][a]);
        }
        cheb_bounds(M, lo, hi);
        for (int e = 0; e < kEnt; ++e) {
            ninc[e] = 0;
            axes[e] = e < 7 ? bits(kDir[e]) : face_axes(e - 7);
        }
        // ascending type, then ascending cube (descending offset bits)
        for (int p = 0; p < 6; ++p) {
            const Kuhn k = kuhn(p);
            for (int ent = 0; ent < 10; ++ent) {
                const int la = ent < 6 ? ent : 12 + 2 * (ent - 6), lb = ent < 6 ? ent + 6 : 13 + 2 * (ent - 6);
                const int pl = plane[p][la], et = pl < 14 ? pl % 7 : 7 + (pl - 14) / 2;
                const int ob = bits(k.vert[low[p][la]]);
                inc[et][ninc[et]++] = p | (ob << 3) | (la << 6) | (lb << 11);
            }
        }
        for (int e = 0; e < kEnt; ++e)
            std::stable_sort(inc[e], inc[e] + ninc[e], [](int x, int y) {
                const int px = x & 7, py = y & 7, ox = (x >> 3) & 7, oy = (y >> 3) & 7;
                return px != py ? px < py : ox > oy;
            });
    }
};
const Ref &ref()
{
    static const Ref r;
    return r;
}

// ------------------------------------------------------------ device side
__constant__ int c2_dof[6][20];          // plane | vertex offset bits << 8
__constant__ double c2_M64[6][400];
__constant__ float c2_M32[6][400];
__constant__ double c2_C[6][20][12];
__constant__ float c2_C32[6][20][12];   // the same, exact in FP32 (dyadic)
__constant__ int c2_ninc[kEnt], c2_inc[kEnt][kMaxInc], c2_axes[kEnt];

struct T2Shot {
    int n[3];
    int pad;
    unsigned long long nnode, ncube, dof0, tet0, ent0;
};

// shot holding flat index i of the per-tetrahedron (which = 0) or
// per-entity (which = 1) ranges
__device__ __forceinline__ int shot_of(const T2Shot *__restrict__ sh, int ns, unsigned long long i, int which)
{
    int lo = 0, hi = ns - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const unsigned long long st = which ? sh[mid].ent0 : sh[mid].tet0;
        if (st <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <class T> __device__ __forceinline__ T mref(int p, int a, int b);
template <> __device__ __forceinline__ double mref<double>(int p, int a, int b) { return c2_M64[p][20 * a + b]; }
template <> __device__ __forceinline__ float mref<float>(int p, int a, int b) { return c2_M32[p][20 * a + b]; }

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

// DOF addressing of flat tetrahedron tl of a shot: DOF a is
// dof0 + plane * nnode + v0 + the vertex offset of its lowest vertex
struct TetAddr {
    int p;
    unsigned long long v0, nx1, nxy, nnode, dof0;
    __device__ __forceinline__ unsigned long long dof(int a) const
    {
        const int d = c2_dof[p][a], ob = d >> 8;
        return dof0 + (unsigned long long)(d & 255) * nnode + v0 + (ob & 1) + ((ob >> 1) & 1) * nx1 + ((ob >> 2) & 1) * nxy;
    }
};
__device__ __forceinline__ TetAddr tet_addr(const T2Shot &S, unsigned long long tl)
{
    TetAddr ta;
    ta.p = (int)(tl / S.ncube);
    const unsigned long long cube = tl - (unsigned long long)ta.p * S.ncube;
    const unsigned long long i = cube % S.n[0], r = cube / S.n[0];
    const unsigned long long j = r % S.n[1], k = r / S.n[1];
    ta.nx1 = S.n[0] + 1;
    ta.nxy = ta.nx1 * (S.n[1] + 1);
    ta.v0 = i + ta.nx1 * j + ta.nxy * k;
    ta.nnode = S.nnode;
    ta.dof0 = S.dof0;
    return ta;
}

// Mass element pass: Yt[a][t] = eps_t (Mref_p x_t)_a (the two-pass
// iteration: this pass, then the entity pass sums the values of an
// entity's tetrahedra).  The type p is dispatched to a compile-time
// constant (tetrahedra are type-major, so a warp holds one type), so the
// reference entries are constant operands of the multiply-adds.
template <class T, int P> __device__ __forceinline__ void mass_elem_body(const TetAddr &ta, unsigned long long NT, unsigned long long t, T e,
                                                                         const T *__restrict__ x, T *__restrict__ Yt)
{
    T xv[20];
#pragma unroll
    for (int b = 0; b < 20; ++b) xv[b] = x[ta.dof(b)];
#pragma unroll
    for (int a = 0; a < 20; ++a) {
        T y = T(0);
#pragma unroll
        for (int b = 0; b < 20; ++b) y = fma(mref<T>(P, a, b), xv[b], y);
        Yt[(unsigned long long)a * NT + t] = mul_rn(e, y);
    }
}

template <class T>
__global__ void __launch_bounds__(128) t2_mass_elem_kernel(unsigned long long NT, const T2Shot *__restrict__ sh, int ns,
                                                          const T *__restrict__ eps, const T *__restrict__ x, T *__restrict__ Yt)
{
    const unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (t >= NT) return;
    const T2Shot S = sh[shot_of(sh, ns, t, 0)];
    const TetAddr ta = tet_addr(S, t - S.tet0);
    const T e = eps[t];
    switch (ta.p) {
    case 0: mass_elem_body<T, 0>(ta, NT, t, e, x, Yt); break;
    case 1: mass_elem_body<T, 1>(ta, NT, t, e, x, Yt); break;
    case 2: mass_elem_body<T, 2>(ta, NT, t, e, x, Yt); break;
    case 3: mass_elem_body<T, 3>(ta, NT, t, e, x, Yt); break;
    case 4: mass_elem_body<T, 4>(ta, NT, t, e, x, Yt); break;
    default: mass_elem_body<T, 5>(ta, NT, t, e, x, Yt); break;
    }
}

// Stiffness element pass in FP64: vertex curls c_v = sum_a U_a C_av, the P1
// mass h_v = (c_v + sum_w c_w) / 120, Yt[a][t] = sum_v C_av . h_v.
template <class TI>
__global__ void __launch_bounds__(128) t2_stiff_elem_kernel(unsigned long long NT, const T2Shot *__restrict__ sh, int ns,
                                                           const TI *__restrict__ U, double *__restrict__ Yt)
{
    const unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (t >= NT) return;
    const T2Shot S = sh[shot_of(sh, ns, t, 0)];
    const TetAddr ta = tet_addr(S, t - S.tet0);
    const int p = ta.p;
    double c[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) c[q] = 0.0;
#pragma unroll 2
    for (int a = 0; a < 20; ++a) {
        const double u = (double)U[ta.dof(a)];
#pragma unroll
        for (int q = 0; q < 12; ++q) c[q] = fma(c2_C[p][a][q], u, c[q]);
    }
    double h[12];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double s = c[q] + c[3 + q] + c[6 + q] + c[9 + q];
#pragma unroll
        for (int v = 0; v < 4; ++v) h[3 * v + q] = (c[3 * v + q] + s) * (1.0 / 120.0);
    }
#pragma unroll 2
    for (int a = 0; a < 20; ++a) {
        double f = 0.0;
#pragma unroll
        for (int q = 0; q < 12; ++q) f = fma(c2_C[p][a][q], h[q], f);
        Yt[(unsigned long long)a * NT + t] = f;
    }
}

// Stiffness element pass of FP32 runs in double-float arithmetic: the same
// vertex curls, P1 mass and transposed curl, each sum a compensated dot
// product (Ogita, Rump and Oishi 2005, Dot2: products split exactly by FMA,
// sums by two-sum, the errors accumulated alongside), so the element values
// carry about twice the FP32 precision at FP32 throughput.  The curl
// coefficients are dyadic (exact in FP32); zero coefficients are skipped
// (the type p is uniform across a warp).
__device__ __forceinline__ void dot2_add(float a, float b, float &s, float &c)
{
    const float p = __fmul_rn(a, b);
    const float ep = fmaf(a, b, -p);
    const float t = __fadd_rn(s, p);
    const float bb = __fsub_rn(t, s);
    const float es = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    s = t;
    c = __fadd_rn(c, __fadd_rn(ep, es));
}

template <int P> __device__ __forceinline__ void stiff_df_body(const TetAddr &ta, unsigned long long NT, unsigned long long t,
                                                               const float *__restrict__ U, double *__restrict__ Yt)
{
    float cs[12], cc[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) { cs[q] = 0.0f; cc[q] = 0.0f; }
#pragma unroll
    for (int a = 0; a < 20; ++a) {
        const float u = U[ta.dof(a)];
#pragma unroll
        for (int q = 0; q < 12; ++q) {
            const float co = c2_C32[P][a][q];
            if (co != 0.0f) dot2_add(co, u, cs[q], cc[q]);
        }
    }
    // P1 mass in FP64 (12 values), split again into hi + lo
    double c[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) c[q] = (double)cs[q] + (double)cc[q];
    float hh[12], hl[12];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double sm = c[q] + c[3 + q] + c[6 + q] + c[9 + q];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const double h = (c[3 * v + q] + sm) * (1.0 / 120.0);
            hh[3 * v + q] = (float)h;
            hl[3 * v + q] = (float)(h - (double)hh[3 * v + q]);
        }
    }
#pragma unroll
    for (int a = 0; a < 20; ++a) {
        float fs = 0.0f, fc = 0.0f;
#pragma unroll
        for (int q = 0; q < 12; ++q) {
            const float co = c2_C32[P][a][q];
            if (co != 0.0f) {
                dot2_add(co, hh[q], fs, fc);
                fc = fmaf(co, hl[q], fc);
            }
        }
        Yt[(unsigned long long)a * NT + t] = (double)fs + (double)fc;
    }
}

__global__ void __launch_bounds__(128, 5) t2_stiff_df_kernel(unsigned long long NT, const T2Shot *__restrict__ sh, int ns,
                                                         const float *__restrict__ U, double *__restrict__ Yt)
{
    const unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (t >= NT) return;
    const T2Shot S = sh[shot_of(sh, ns, t, 0)];
    const TetAddr ta = tet_addr(S, t - S.tet0);
    switch (ta.p) {
    case 0: stiff_df_body<0>(ta, NT, t, U, Yt); break;
    case 1: stiff_df_body<1>(ta, NT, t, U, Yt); break;
    case 2: stiff_df_body<2>(ta, NT, t, U, Yt); break;
    case 3: stiff_df_body<3>(ta, NT, t, U, Yt); break;
    case 4: stiff_df_body<4>(ta, NT, t, U, Yt); break;
    default: stiff_df_body<5>(ta, NT, t, U, Yt); break;
    }
}

enum { G_FORCE = 0, G_KICK = 1, G_CHEB0 = 2, G_CHEB = 3 };
enum { FIN_NONE = 0, FIN_DRIFT = 1, FIN_LEAP = 2 };

template <class T> struct GArgs {
    const void *Yt;
    unsigned long long NT;
    double *P;       // momentum (FP64 in both precisions)
    T *Pc;           // P in the run precision (FP32 runs), the right-hand side of the solve
    T *out;          // G_FORCE output
    const T *b;      // right-hand side of the solve
    T *x, *d;        // Chebyshev iterate (written) and step
    const T *xin;    // Chebyshev iterate read by the fused mass rows (G_CHEB)
    const T *eps;    // permittivity per tetrahedron (G_CHEB)
    const T *pinv;   // 2 x 2 block inverses, three planes over the entities
    T *U, *Uold;
    double a;        // kick: P -= a F
    double h;        // final iteration: U += h x (drift) or U = 2U - Uold - h x (leapfrog)
    double c0, c1, c2;   // Chebyshev: d = c1 d + c2 z (c0 = 1 / theta for the first step)
};

// Entity pass: one thread per edge or face of a node (both its DOFs).  Sums
// the element values of its tetrahedra in the fixed order of c2_inc, then
// applies the mode's update.  Unused and boundary-tangential entities are
// held at zero.
template <class T, class TY, int MODE, int FIN>
__global__ void __launch_bounds__(128) t2_gather_kernel(unsigned long long NE, const T2Shot *__restrict__ sh, int ns, GArgs<T> g)
{
    const unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (e >= NE) return;
    const T2Shot S = sh[shot_of(sh, ns, e, 1)];
    const unsigned long long el = e - S.ent0;
    const int et = (int)(el / S.nnode);
    const unsigned long long v = el - (unsigned long long)et * S.nnode;
    const int nx1 = S.n[0] + 1, ny1 = S.n[1] + 1;
    const int i = (int)(v % nx1), j = (int)((v / nx1) % ny1), k = (int)(v / ((unsigned long long)nx1 * ny1));
    const int x3[3] = {i, j, k};
    const int ax = c2_axes[et];
    bool dead = false;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int in = (ax >> q) & 1;
        if (x3[q] + in > S.n[q]) dead = true;
        if (!in && (x3[q] == 0 || x3[q] == S.n[q])) dead = true;
    }
    const int pl0 = et < 7 ? et : 14 + 2 * (et - 7), pl1 = et < 7 ? et + 7 : pl0 + 1;
    const unsigned long long d0 = S.dof0 + (unsigned long long)pl0 * S.nnode + v;
    const unsigned long long d1 = S.dof0 + (unsigned long long)pl1 * S.nnode + v;
    TY y0 = TY(0), y1 = TY(0);
    if (MODE != G_CHEB0 && !dead) {
        // every value of the entity's tetrahedra loaded first (all loads in
        // flight together), then summed in the fixed order of c2_inc
        const TY *Y = static_cast<const TY *>(g.Yt);
        const unsigned long long ncx = S.n[0], ncxy = ncx * S.n[1];
        const int ninc = c2_ninc[et];
        TY v0[kMaxInc], v1[kMaxInc];
        bool in[kMaxInc];
#pragma unroll
        for (int q = 0; q < kMaxInc; ++q) {
            in[q] = false;
            v0[q] = v1[q] = TY(0);
            if (q >= ninc) continue;
            const int w = c2_inc[et][q];
            const int p = w & 7, ob = (w >> 3) & 7, la = (w >> 6) & 31, lb = (w >> 11) & 31;
            const int ci = i - (ob & 1), cj = j - ((ob >> 1) & 1), ck = k - ((ob >> 2) & 1);
            if (ci < 0 || cj < 0 || ck < 0 || ci >= S.n[0] || cj >= S.n[1] || ck >= S.n[2]) continue;
            const unsigned long long t = S.tet0 + (unsigned long long)p * S.ncube + (unsigned long long)ci + ncx * cj + ncxy * ck;
            in[q] = true;
            v0[q] = Y[(unsigned long long)la * g.NT + t];
            v1[q] = Y[(unsigned long long)lb * g.NT + t];
        }
#pragma unroll
        for (int q = 0; q < kMaxInc; ++q)
            if (in[q]) {
                y0 = add_rn(y0, v0[q]);
                y1 = add_rn(y1, v1[q]);
            }
    }
    if (MODE == G_FORCE) {
        g.out[d0] = dead ? T(0) : (T)y0;
        g.out[d1] = dead ? T(0) : (T)y1;
        return;
    }
    if (MODE == G_KICK) {
        if (dead) return;
        const double p0 = g.P[d0] - g.a * (double)y0, p1 = g.P[d1] - g.a * (double)y1;
        g.P[d0] = p0; g.P[d1] = p1;
        if (g.Pc) { g.Pc[d0] = (T)p0; g.Pc[d1] = (T)p1; }
        return;
    }
    // Chebyshev: r = b - M x, z = Pinv r, d = c1 d + c2 z (first: d = z / theta), x += d
    if (dead) {
        g.x[d0] = T(0); g.x[d1] = T(0); g.d[d0] = T(0); g.d[d1] = T(0);
        return;
    }
    const T r0 = g.b[d0] - (T)y0, r1 = g.b[d1] - (T)y1;
    const T q00 = g.pinv[e], q01 = g.pinv[NE + e], q11 = g.pinv[2 * NE + e];
    const T z0 = fma(q00, r0, q01 * r1), z1 = fma(q01, r0, q11 * r1);
    T n0, n1, x0, x1;
    if (MODE == G_CHEB0) {
        n0 = (T)g.c0 * z0; n1 = (T)g.c0 * z1;
        x0 = n0; x1 = n1;
    } else {
        n0 = fma((T)g.c1, g.d[d0], (T)g.c2 * z0);
        n1 = fma((T)g.c1, g.d[d1], (T)g.c2 * z1);
        x0 = g.xin[d0] + n0; x1 = g.xin[d1] + n1;   // the two-pass iteration reads and writes the same buffer
    }
    g.d[d0] = n0; g.d[d1] = n1;
    g.x[d0] = x0; g.x[d1] = x1;
    if (FIN == FIN_DRIFT) {
        g.U[d0] = fma((T)g.h, x0, g.U[d0]);
        g.U[d1] = fma((T)g.h, x1, g.U[d1]);
    } else if (FIN == FIN_LEAP) {
        const T u0 = g.U[d0], u1 = g.U[d1];
        g.U[d0] = fma(-(T)g.h, x0, T(2) * u0 - g.Uold[d0]);
        g.U[d1] = fma(-(T)g.h, x1, T(2) * u1 - g.Uold[d1]);
        g.Uold[d0] = u0; g.Uold[d1] = u1;
    }
}

// ------------------------------------------- compile-time incidence tables
// The incidences of the 19 entity types and the DOF placement of the six
// tetrahedron types follow from the Kuhn split alone, so they are built at
// compile time for the fused iteration (the same tables as Ref, whose
// element matrices need floating-point setup and stay in constant memory).
struct IncTab {
    int n[kEnt];
    int p[kEnt][kMaxInc], ob[kEnt][kMaxInc], la[kEnt][kMaxInc], lb[kEnt][kMaxInc];
    int plane[6][20], vo[6][20];   // plane and lowest-vertex offset bits of local DOF b of type p
};

constexpr int cx_dir(int dx, int dy, int dz)
{
    for (int k = 0; k < 7; ++k)
        if (kDir[k][0] == dx && kDir[k][1] == dy && kDir[k][2] == dz) return k;
    return -1;
}
constexpr int cx_face(int s1, int s2)
{
    int t = 0;
    for (int a = 1; a < 8; ++a)
        for (int b = 1; b < 8; ++b) {
            if (a & b) continue;
            if (a == s1 && b == s2) return t;
            ++t;
        }
    return -1;
}

constexpr IncTab make_inc_tab()
{
    IncTab T{};
    int vert[6][4][3] = {};
    for (int p = 0; p < 6; ++p) {
        const int a = kPerm[p][0], b = kPerm[p][1];
        vert[p][1][a] = 1;
        vert[p][2][a] = 1; vert[p][2][b] = 1;
        vert[p][3][0] = vert[p][3][1] = vert[p][3][2] = 1;
        for (int d = 0; d < 20; ++d) {
            int low = 0, plane = 0;
            if (d < 12) {
                const int l = d % 6, i = kEdge[l][0], j = kEdge[l][1];
                plane = cx_dir(vert[p][j][0] - vert[p][i][0], vert[p][j][1] - vert[p][i][1], vert[p][j][2] - vert[p][i][2]) + (d < 6 ? 0 : 7);
                low = i;
            } else {
                const int f = (d - 12) / 2, v0 = kFace[f][0], v1 = kFace[f][1], v2 = kFace[f][2];
                int s1 = 0, s2 = 0;
                for (int q = 0; q < 3; ++q) {
                    s1 |= (vert[p][v1][q] - vert[p][v0][q]) << q;
                    s2 |= (vert[p][v2][q] - vert[p][v1][q]) << q;
                }
                plane = 14 + 2 * cx_face(s1, s2) + (d - 12) % 2;
                low = v0;
            }
            T.plane[p][d] = plane;
            T.vo[p][d] = vert[p][low][0] | (vert[p][low][1] << 1) | (vert[p][low][2] << 2);
        }
    }
    for (int p = 0; p < 6; ++p)
        for (int ent = 0; ent < 10; ++ent) {
            const int la = ent < 6 ? ent : 12 + 2 * (ent - 6), lb = ent < 6 ? ent + 6 : 13 + 2 * (ent - 6);
            const int pl = T.plane[p][la], et = pl < 14 ? pl % 7 : 7 + (pl - 14) / 2;
            const int q = T.n[et]++;
            T.p[et][q] = p; T.ob[et][q] = T.vo[p][la]; T.la[et][q] = la; T.lb[et][q] = lb;
        }
    // ascending type, then ascending cube (descending offset bits), as Ref
    for (int e = 0; e < kEnt; ++e)
        for (int a = 1; a < T.n[e]; ++a)
            for (int b = a; b > 0; --b) {
                const bool swap = T.p[e][b - 1] > T.p[e][b] || (T.p[e][b - 1] == T.p[e][b] && T.ob[e][b - 1] < T.ob[e][b]);
                if (!swap) break;
                int t = 0;
                t = T.p[e][b]; T.p[e][b] = T.p[e][b - 1]; T.p[e][b - 1] = t;
                t = T.ob[e][b]; T.ob[e][b] = T.ob[e][b - 1]; T.ob[e][b - 1] = t;
                t = T.la[e][b]; T.la[e][b] = T.la[e][b - 1]; T.la[e][b - 1] = t;
                t = T.lb[e][b]; T.lb[e][b] = T.lb[e][b - 1]; T.lb[e][b - 1] = t;
            }
    return T;
}
constexpr IncTab kInc = make_inc_tab();
static_assert(kInc.n[6] == 6 && kInc.n[7] == 2, "Kuhn split: the body diagonal lies in six tetrahedra, a face in two");

// The two mass rows of entity type ET at node (i,j,k): sum over its
// tetrahedra of eps_t (Mref_p x_t) at the entity's local DOFs, every table
// entry a compile-time constant (the reference entries are constant-bank
// operands, the DOF offsets plane * nnode + vertex offset).
// r0 += Mref_p[LA][b] x_b, r1 += Mref_p[LB][b] x_b over b in order, the DOF
// offset of b (plane * nnode + vertex offset) formed from compile-time parts
template <class T, int P, int LA, int LB, int B>
__device__ __forceinline__ void cheb_term(const T *__restrict__ xs, unsigned nn, unsigned nx1, unsigned nxy, T &r0, T &r1)
{
    constexpr int PL = kInc.plane[P][B], VO = kInc.vo[P][B];
    const T xb = xs[(unsigned)PL * nn + (VO & 1) + ((VO >> 1) & 1) * nx1 + ((VO >> 2) & 1) * nxy];
    r0 = fma(mref<T>(P, LA, B), xb, r0);
    r1 = fma(mref<T>(P, LB, B), xb, r1);
}
template <class T, int P, int LA, int LB, int... B>
__device__ __forceinline__ void cheb_terms(std::integer_sequence<int, B...>, const T *__restrict__ xs, unsigned nn, unsigned nx1,
                                           unsigned nxy, T &r0, T &r1)
{
    (cheb_term<T, P, LA, LB, B>(xs, nn, nx1, nxy, r0, r1), ...);
}

template <class T, int ET, int Q>
__device__ __forceinline__ void cheb_rows_inc(const T *__restrict__ xs, const T *__restrict__ eps, unsigned long long tet0,
                                              unsigned ncube, unsigned nn, unsigned nx1, unsigned nxy, unsigned ncx, unsigned ncxy,
                                              const int (&n)[3], int i, int j, int k, T &y0, T &y1)
{
    constexpr int P = kInc.p[ET][Q], OB = kInc.ob[ET][Q], LA = kInc.la[ET][Q], LB = kInc.lb[ET][Q];
    const int ci = i - (OB & 1), cj = j - ((OB >> 1) & 1), ck = k - ((OB >> 2) & 1);
    if (ci < 0 || cj < 0 || ck < 0 || ci >= n[0] || cj >= n[1] || ck >= n[2]) return;
    const unsigned v0 = (unsigned)ci + nx1 * cj + nxy * ck;
    T r0 = T(0), r1 = T(0);
    cheb_terms<T, P, LA, LB>(std::make_integer_sequence<int, 20>{}, xs + v0, nn, nx1, nxy, r0, r1);
    // the rounded product, then the rounded sum: the two-pass form stores
    // e * r and sums the stored values in the same order, so both forms give
    // the same bits
    const T e = eps[tet0 + (unsigned long long)P * ncube + (unsigned)ci + ncx * cj + ncxy * ck];
    y0 = add_rn(y0, mul_rn(e, r0));
    y1 = add_rn(y1, mul_rn(e, r1));
}

template <class T, int ET, int... Q>
__device__ __forceinline__ void cheb_rows_all(std::integer_sequence<int, Q...>, const T *__restrict__ xs, const T *__restrict__ eps,
                                              unsigned long long tet0, unsigned ncube, unsigned nn, unsigned nx1, unsigned nxy,
                                              unsigned ncx, unsigned ncxy, const int (&n)[3], int i, int j, int k, T &y0, T &y1)
{
    (cheb_rows_inc<T, ET, Q>(xs, eps, tet0, ncube, nn, nx1, nxy, ncx, ncxy, n, i, j, k, y0, y1), ...);
}

template <class T, int ET>
__device__ __forceinline__ void cheb_rows(const T *__restrict__ xs, const T *__restrict__ eps, unsigned long long tet0, unsigned ncube,
                                          unsigned nn, unsigned nx1, unsigned nxy, unsigned ncx, unsigned ncxy, const int (&n)[3], int i,
                                          int j, int k, T &y0, T &y1)
{
    cheb_rows_all<T, ET>(std::make_integer_sequence<int, kInc.n[ET]>{}, xs, eps, tet0, ncube, nn, nx1, nxy, ncx, ncxy, n, i, j, k, y0,
                         y1);
}

// Fused Chebyshev iteration: one thread per edge or face forms the entity's
// two mass rows eps_t (Mref_p x_t) over its tetrahedra (fixed order) from
// the previous iterate, then r = b - M x, z = Pinv r, d = c1 d + c2 z and
// the next iterate x + d into the other buffer.  The entity type selects a
// body compiled for its incidences (cheb_rows); the entity types are
// plane-major, so a warp holds one type.
template <class T, int FIN>
__global__ void __launch_bounds__(128) t2_cheb_kernel(unsigned long long NE, const T2Shot *__restrict__ sh, int ns, GArgs<T> g)
{
    const unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (e >= NE) return;
    const T2Shot S = sh[shot_of(sh, ns, e, 1)];
    const unsigned nn = (unsigned)S.nnode;
    const unsigned el = (unsigned)(e - S.ent0);
    const int et = (int)(el / nn);
    const unsigned v = el - (unsigned)et * nn;
    const unsigned nx1 = S.n[0] + 1, ny1 = S.n[1] + 1;
    const int i = (int)(v % nx1), j = (int)((v / nx1) % ny1), k = (int)(v / (nx1 * ny1));
    const int x3[3] = {i, j, k};
    const int ax = c2_axes[et];
    bool dead = false;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int in = (ax >> q) & 1;
        if (x3[q] + in > S.n[q]) dead = true;
        if (!in && (x3[q] == 0 || x3[q] == S.n[q])) dead = true;
    }
    const int pl0 = et < 7 ? et : 14 + 2 * (et - 7), pl1 = et < 7 ? et + 7 : pl0 + 1;
    const unsigned long long d0 = S.dof0 + (unsigned long long)pl0 * nn + v;
    const unsigned long long d1 = S.dof0 + (unsigned long long)pl1 * nn + v;
    if (dead) {
        g.x[d0] = T(0); g.x[d1] = T(0); g.d[d0] = T(0); g.d[d1] = T(0);
        return;
    }
    const T *xs = g.xin + S.dof0;
    const unsigned ncx = S.n[0], ncxy = ncx * S.n[1], nxy = nx1 * ny1;
    const int n3[3] = {S.n[0], S.n[1], S.n[2]};
    const unsigned nc = (unsigned)S.ncube;
    T y0 = T(0), y1 = T(0);
#define EMS_T2_ROWS(E) \
    case E: cheb_rows<T, E>(xs, g.eps, S.tet0, nc, nn, nx1, nxy, ncx, ncxy, n3, i, j, k, y0, y1); break;
    switch (et) {
        EMS_T2_ROWS(0) EMS_T2_ROWS(1) EMS_T2_ROWS(2) EMS_T2_ROWS(3) EMS_T2_ROWS(4) EMS_T2_ROWS(5) EMS_T2_ROWS(6)
        EMS_T2_ROWS(7) EMS_T2_ROWS(8) EMS_T2_ROWS(9) EMS_T2_ROWS(10) EMS_T2_ROWS(11) EMS_T2_ROWS(12) EMS_T2_ROWS(13)
        EMS_T2_ROWS(14) EMS_T2_ROWS(15) EMS_T2_ROWS(16) EMS_T2_ROWS(17) default: EMS_T2_ROWS(18)
    }
#undef EMS_T2_ROWS
    const T r0 = g.b[d0] - y0, r1 = g.b[d1] - y1;
    const T q00 = g.pinv[e], q01 = g.pinv[NE + e], q11 = g.pinv[2 * NE + e];
    const T z0 = fma(q00, r0, q01 * r1), z1 = fma(q01, r0, q11 * r1);
    const T n0 = fma((T)g.c1, g.d[d0], (T)g.c2 * z0), n1 = fma((T)g.c1, g.d[d1], (T)g.c2 * z1);
    const T x0 = g.xin[d0] + n0, x1 = g.xin[d1] + n1;
    g.d[d0] = n0; g.d[d1] = n1;
    g.x[d0] = x0; g.x[d1] = x1;
    if (FIN == FIN_DRIFT) {
        g.U[d0] = fma((T)g.h, x0, g.U[d0]);
        g.U[d1] = fma((T)g.h, x1, g.U[d1]);
    } else if (FIN == FIN_LEAP) {
        const T u0 = g.U[d0], u1 = g.U[d1];
        g.U[d0] = fma(-(T)g.h, x0, T(2) * u0 - g.Uold[d0]);
        g.U[d1] = fma(-(T)g.h, x1, T(2) * u1 - g.Uold[d1]);
        g.Uold[d0] = u0; g.Uold[d1] = u1;
    }
}

// 2 x 2 block inverse per entity from the assembled eps-weighted mass (FP64).
__global__ void __launch_bounds__(128) t2_pinv_kernel(unsigned long long NE, const T2Shot *__restrict__ sh, int ns,
                                                      const double *__restrict__ eps, double *__restrict__ out)
{
    const unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (e >= NE) return;
    const T2Shot S = sh[shot_of(sh, ns, e, 1)];
    const unsigned long long el = e - S.ent0;
    const int et = (int)(el / S.nnode);
    const unsigned long long v = el - (unsigned long long)et * S.nnode;
    const int nx1 = S.n[0] + 1, ny1 = S.n[1] + 1;
    const int i = (int)(v % nx1), j = (int)((v / nx1) % ny1), k = (int)(v / ((unsigned long long)nx1 * ny1));
    double a = 0.0, b = 0.0, c = 0.0;
    const unsigned long long ncx = S.n[0], ncxy = ncx * S.n[1];
    for (int q = 0; q < c2_ninc[et]; ++q) {
        const int w = c2_inc[et][q];
        const int p = w & 7, ob = (w >> 3) & 7, la = (w >> 6) & 31, lb = (w >> 11) & 31;
        const int ci = i - (ob & 1), cj = j - ((ob >> 1) & 1), ck = k - ((ob >> 2) & 1);
        if (ci < 0 || cj < 0 || ck < 0 || ci >= S.n[0] || cj >= S.n[1] || ck >= S.n[2]) continue;
        const double ep = eps[S.tet0 + (unsigned long long)p * S.ncube + (unsigned long long)ci + ncx * cj + ncxy * ck];
        a += ep * c2_M64[p][21 * la];
        b += ep * c2_M64[p][20 * la + lb];
        c += ep * c2_M64[p][21 * lb];
    }
    const double det = a * c - b * b;
    const bool ok = a > 0.0 && det > 0.0;
    out[e] = ok ? c / det : 0.0;
    out[NE + e] = ok ? -b / det : 0.0;
    out[2 * NE + e] = ok ? a / det : 0.0;
}

template <class T> __global__ void t2_narrow_kernel(unsigned long long n, const double *__restrict__ x, T *__restrict__ y)
{
    const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i < n) y[i] = (T)x[i];
}

template <class T> __global__ void t2_axpy_kernel(unsigned long long n, T *__restrict__ U, const T *__restrict__ x, double h)
{
    const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i < n) U[i] = fma((T)h, x[i], U[i]);
}

// Dipole loads, one thread per loaded DOF (its entries in dipole order):
// symplectic P += s sum_k coef_k g_k (and the run-precision copy), leapfrog
// b -= sum_k coef_k g_k.
template <class T, int LEAP>
__global__ void t2_source_kernel(int n, const unsigned long long *__restrict__ dof, const int *__restrict__ ptr,
                                 const int *__restrict__ dip, const double *__restrict__ coef, const double *__restrict__ gt,
                                 const int *__restrict__ ctl, int nsub, int q, int nd, double s, double *__restrict__ P,
                                 T *__restrict__ vec)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double *g = gt + ((size_t)ctl[0] * nsub + q) * nd;
    double f = 0.0;
    for (int j = ptr[k]; j < ptr[k + 1]; ++j) f += coef[j] * g[dip[j]];
    const unsigned long long e = dof[k];
    if (LEAP) {
        vec[e] = (T)((double)vec[e] - f);
    } else {
        const double p = P[e] + s * f;
        P[e] = p;
        if (vec) vec[e] = (T)p;
    }
}

// Receivers: one warp each; lane a < 20 forms its function's terms, a fixed
// shuffle tree sums them.
template <class T>
__global__ void t2_sample_kernel(int nrec, const unsigned long long *__restrict__ rdof, const double *__restrict__ rw,
                                 const T *__restrict__ U, const int *__restrict__ ctl, int tf, int nsamp, double *__restrict__ tr)
{
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), l = threadIdx.x & 31;
    const int step = ctl[0];
    if (r >= nrec || step % tf != 0 || step / tf >= nsamp) return;
    double c[3] = {0.0, 0.0, 0.0};
    if (l < 20) {
        const double u = (double)U[rdof[20 * r + l]];
        for (int q = 0; q < 3; ++q) c[q] = u * rw[60 * r + 3 * l + q];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        for (int q = 0; q < 3; ++q) c[q] += __shfl_down_sync(0xffffffffu, c[q], o);
    if (l == 0) {
        double *o = tr + ((size_t)r * nsamp + step / tf) * 4;
        o[1] = c[0]; o[2] = c[1]; o[3] = c[2];
    }
}

__global__ void t2_advance_kernel(int *ctl) { ctl[0] += 1; }

// Block partial sums of x . y (fixed grid, fixed order); the host adds them.
template <class T>
__global__ void __launch_bounds__(256) t2_dot_kernel(unsigned long long n, const T *__restrict__ x, const T *__restrict__ y,
                                                    double *__restrict__ part)
{
    __shared__ double sm[256];
    double s = 0.0;
    for (unsigned long long i = blockIdx.x * 256ull + threadIdx.x; i < n; i += 256ull * gridDim.x) s += (double)x[i] * (double)y[i];
    sm[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

template <class T> __global__ void t2_scale_kernel(unsigned long long n, T *__restrict__ x, double s)
{
    const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i < n) x[i] = (T)((double)x[i] * s);
}

// Gradient contraction of the adjoint: grad_t += c * Z_t . (Mref_p Y_t), the
// element product in the run precision, the sum over time in FP64.
template <class T>
__global__ void __launch_bounds__(128) t2_grad_kernel(unsigned long long NT, const T2Shot *__restrict__ sh, int ns,
                                                     const T *__restrict__ Z, const T *__restrict__ Y, double c,
                                                     double *__restrict__ grad)
{
    const unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (t >= NT) return;
    const T2Shot S = sh[shot_of(sh, ns, t, 0)];
    const TetAddr ta = tet_addr(S, t - S.tet0);
    T yv[20];
#pragma unroll
    for (int b = 0; b < 20; ++b) yv[b] = Y[ta.dof(b)];
    const int p = ta.p;
    T s = T(0);
#pragma unroll 4
    for (int a = 0; a < 20; ++a) {
        T r = T(0);
#pragma unroll
        for (int b = 0; b < 20; ++b) r = fma(mref<T>(p, a, b), yv[b], r);
        s = fma(Z[ta.dof(a)], r, s);
    }
    grad[t] += c * (double)s;
}

__global__ void t2_set_kernel(int *p, int v) { *p = v; }

constexpr int kDotBlocks = 512;

unsigned blocks(unsigned long long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

// ---------------------------------------------------------------- host side
struct Tet2Sim : Sim {
    struct ShotH {
        int n[3];
        size_t nnode, ncube, dof0, tet0, ent0;
    };
    struct Dip {
        size_t dof[20];
        double coef[20];
        int kind;
        double f0n;
    };
    ems_tetfem_params P;
    std::vector<ShotH> shots;
    size_t ndof = 0, ntet = 0, nent = 0;
    bool fp64 = false, ready = false, y_valid = false;
    double c0 = 299792458.0, tscale = 1.0, dtn = 0.0, dt_lim_n = 0.0, lambda_max = 0.0, cur_time = 0.0;
    int mass_iters = kMassIters;
    std::vector<double> eps_h;   // API order per shot: 6 * cell + p
    std::vector<Dip> dips;
    std::vector<std::array<size_t, 20>> rec_dof;
    std::vector<std::array<double, 60>> rec_w;
    DevBuf d_shots, d_eps, d_pinv, d_U, d_Uold, d_P, d_Pc, d_x, d_xs, d_d, d_b, d_YtM, d_YtK, d_ctl, d_part;
    DevBuf d_src_dof, d_src_ptr, d_src_dip, d_src_coef, d_src_g, d_rec_dof, d_rec_w, d_tr;
    std::vector<double> cheb_c1, cheb_c2;
    double cheb_c0 = 0.0;
    // adjoint: snapshots of (U, P) at segment starts of the recorded run
    int ckpt_nsnap = 0, rec_nsteps = -1, rec_seg = 0;
    DevBuf d_snap;

    Tet2Sim(const ems_tetfem_params *p, const std::vector<std::array<int, 3>> &cells) : Sim(Kind::TETFEM), P(*p)
    {
        EMS_CHECK_ARG(!cells.empty(), "at least one shot");
        size_t n0 = 0, t0 = 0, e0 = 0;
        for (auto &c : cells) {
            EMS_CHECK_ARG(c[0] > 0 && c[1] > 0 && c[2] > 0, "cell counts must be positive");
            ShotH s{};
            s.n[0] = c[0]; s.n[1] = c[1]; s.n[2] = c[2];
            s.nnode = (size_t)(c[0] + 1) * (c[1] + 1) * (c[2] + 1);
            s.ncube = (size_t)c[0] * c[1] * c[2];
            s.dof0 = n0; s.tet0 = t0; s.ent0 = e0;
            n0 += kPlanes * s.nnode;
            t0 += 6 * s.ncube;
            e0 += kEnt * s.nnode;
            shots.push_back(s);
        }
        EMS_CHECK_ARG(P.h > 0, "h must be positive");
        EMS_CHECK_ARG(P.integrator == EMS_LEAPFROG || P.integrator == EMS_SYMP2 || P.integrator == EMS_SYMP4,
                      "tetrahedral integrator must be EMS_LEAPFROG, EMS_SYMP2 or EMS_SYMP4");
        EMS_CHECK_ARG(P.precision == EMS_FP64 || P.precision == EMS_FP32, "precision must be EMS_FP64 or EMS_FP32");
        EMS_CHECK_ARG(P.dt >= 0 && P.time_frequency > 0, "dt must be >= 0 and time_frequency > 0");
        if (P.cfl_fraction <= 0) P.cfl_fraction = 0.9;
        EMS_CHECK_ARG(P.cfl_fraction < 1.0, "cfl_fraction must be below 1");
        fp64 = P.precision == EMS_FP64;
        tscale = P.h / c0;
        ndof = n0; ntet = t0; nent = e0;
        EMS_CHECK_ARG(ndof < (size_t)1 << 40, "mesh too large");
        eps_h.assign(ntet, 1.0);
        init_stream();
        upload_tables();
        std::vector<T2Shot> sh(shots.size());
        for (size_t s = 0; s < shots.size(); ++s) {
            for (int q = 0; q < 3; ++q) sh[s].n[q] = shots[s].n[q];
            sh[s].nnode = shots[s].nnode; sh[s].ncube = shots[s].ncube;
            sh[s].dof0 = shots[s].dof0; sh[s].tet0 = shots[s].tet0; sh[s].ent0 = shots[s].ent0;
        }
        d_shots.alloc(sh.size() * sizeof(T2Shot));
        EMS_CUDA(cudaMemcpy(d_shots.p, sh.data(), sh.size() * sizeof(T2Shot), cudaMemcpyHostToDevice));
        for (const ShotH &S : shots)
            EMS_CHECK_ARG(kPlanes * S.nnode < ((size_t)1 << 32), "shot too large for 32-bit DOF offsets");
        const size_t w = fp64 ? 8 : 4;
        d_U.alloc(ndof * w); d_Uold.alloc(ndof * w); d_P.alloc(ndof * 8);
        d_x.alloc(ndof * w); d_xs.alloc(ndof * w); d_d.alloc(ndof * w); d_b.alloc(ndof * w);
        if (!fp64) d_Pc.alloc(ndof * 4);
        d_YtM.alloc(20 * ntet * w);
        d_YtK.alloc(20 * ntet * 8);
        d_ctl.alloc(16);
        d_part.alloc(kDotBlocks * 8);
        reset();
    }

    static void upload_tables()
    {
        const Ref &R = ref();
        // the fused iteration's compile-time tables must be the setup's
        for (int e = 0; e < kEnt; ++e) {
            bool same = kInc.n[e] == R.ninc[e];
            for (int q = 0; same && q < R.ninc[e]; ++q) {
                const int w = R.inc[e][q];
                same = kInc.p[e][q] == (w & 7) && kInc.ob[e][q] == ((w >> 3) & 7) && kInc.la[e][q] == ((w >> 6) & 31) &&
                       kInc.lb[e][q] == ((w >> 11) & 31);
            }
            if (!same) throw Error{EMS_ERR_CUDA, "compile-time incidence table differs from the setup's"};
        }
        for (int p = 0; p < 6; ++p) {
            const Kuhn k = kuhn(p);
            for (int a = 0; a < 20; ++a)
                if (kInc.plane[p][a] != R.plane[p][a] || kInc.vo[p][a] != bits(k.vert[R.low[p][a]]))
                    throw Error{EMS_ERR_CUDA, "compile-time DOF table differs from the setup's"};
        }
        int dof[6][20];
        float m32[6][400];
        for (int p = 0; p < 6; ++p) {
            const Kuhn k = kuhn(p);
            for (int a = 0; a < 20; ++a) dof[p][a] = R.plane[p][a] | (bits(k.vert[R.low[p][a]]) << 8);
            for (int q = 0; q < 400; ++q) m32[p][q] = (float)R.M[p][q];
        }
        EMS_CUDA(cudaMemcpyToSymbol(c2_dof, dof, sizeof(dof)));
        EMS_CUDA(cudaMemcpyToSymbol(c2_M64, R.M, sizeof(R.M)));
        EMS_CUDA(cudaMemcpyToSymbol(c2_M32, m32, sizeof(m32)));
        EMS_CUDA(cudaMemcpyToSymbol(c2_C, R.C, sizeof(R.C)));
        float c32[6][20][12];
        for (int p = 0; p < 6; ++p)
            for (int a = 0; a < 20; ++a)
                for (int q = 0; q < 12; ++q) {
                    c32[p][a][q] = (float)R.C[p][a][q];
                    if ((double)c32[p][a][q] != R.C[p][a][q]) throw Error{EMS_ERR_CUDA, "curl coefficient not exact in FP32"};
                }
        EMS_CUDA(cudaMemcpyToSymbol(c2_C32, c32, sizeof(c32)));
        EMS_CUDA(cudaMemcpyToSymbol(c2_ninc, R.ninc, sizeof(R.ninc)));
        EMS_CUDA(cudaMemcpyToSymbol(c2_inc, R.inc, sizeof(R.inc)));
        EMS_CUDA(cudaMemcpyToSymbol(c2_axes, R.axes, sizeof(R.axes)));
    }

    // API position (6 * cell + p within a shot) -> type-major device order
    size_t tet_index(size_t api) const
    {
        size_t s = shots.size() - 1;
        while (shots[s].tet0 > api) --s;
        const size_t l = api - shots[s].tet0, cell = l / 6, p = l % 6;
        return shots[s].tet0 + p * shots[s].ncube + cell;
    }
    // API DOF (38 * node + plane within a shot) -> device plane layout
    size_t dof_index(size_t api) const
    {
        size_t s = shots.size() - 1;
        while (shots[s].dof0 > api) --s;
        const size_t l = api - shots[s].dof0, node = l / kPlanes, pl = l % kPlanes;
        return shots[s].dof0 + pl * shots[s].nnode + node;
    }

    void set_material(const double *eps_r, const double *sigma)
    {
        EMS_CHECK_ARG(eps_r != nullptr, "eps_r required");
        for (size_t t = 0; t < ntet; ++t) EMS_CHECK_ARG(eps_r[t] > 0 && std::isfinite(eps_r[t]), "eps_r must be positive");
        if (sigma)
            for (size_t t = 0; t < ntet; ++t)
                if (sigma[t] != 0.0) throw Error{EMS_ERR_UNSUPPORTED, "conductivity is implemented for order-1 tetrahedra only"};
        eps_h.assign(eps_r, eps_r + ntet);
        ready = false;
        y_valid = false;
        rec_nsteps = -1;
    }

    template <class T> void launch_pinv_and_eps()
    {
        std::vector<double> e(ntet);
        for (size_t t = 0; t < ntet; ++t) e[tet_index(t)] = eps_h[t];
        DevBuf e64, p64;
        e64.alloc(ntet * 8);
        p64.alloc(3 * nent * 8);
        EMS_CUDA(cudaMemcpy(e64.p, e.data(), ntet * 8, cudaMemcpyHostToDevice));
        t2_pinv_kernel<<<blocks(nent, 128), 128, 0, stream>>>(nent, d_shots.as<T2Shot>(), (int)shots.size(), e64.as<double>(),
                                                              p64.as<double>());
        d_eps.ensure(ntet * sizeof(T));
        d_pinv.ensure(3 * nent * sizeof(T));
        t2_narrow_kernel<T><<<blocks(ntet, 256), 256, 0, stream>>>(ntet, e64.as<double>(), d_eps.as<T>());
        t2_narrow_kernel<T><<<blocks(3 * nent, 256), 256, 0, stream>>>(3 * nent, p64.as<double>(), d_pinv.as<T>());
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    void cheb_coefficients()
    {
        const Ref &R = ref();
        const double th = 0.5 * (R.hi + R.lo), de = 0.5 * (R.hi - R.lo), sg = th / de;
        double rho = 1.0 / sg;
        cheb_c0 = 1.0 / th;
        cheb_c1.assign(mass_iters, 0.0);
        cheb_c2.assign(mass_iters, 0.0);
        for (int k = 1; k < mass_iters; ++k) {
            const double rn = 1.0 / (2.0 * sg - rho);
            cheb_c1[k] = rn * rho;
            cheb_c2[k] = 2.0 * rn / de;
            rho = rn;
        }
    }

    template <class T> GArgs<T> gargs() const
    {
        GArgs<T> g{};
        g.NT = ntet;
        g.P = d_P.as<double>();
        g.Pc = fp64 ? nullptr : reinterpret_cast<T *>(d_Pc.p);
        g.pinv = d_pinv.as<T>();
        g.x = d_x.as<T>(); g.d = d_d.as<T>();
        g.U = d_U.as<T>(); g.Uold = d_Uold.as<T>();
        return g;
    }
    template <class T> const T *rhs_P() const { return fp64 ? reinterpret_cast<const T *>(d_P.p) : reinterpret_cast<const T *>(d_Pc.p); }

    // Stiffness element pass into d_YtK: FP64 for FP64 runs, double-float for FP32
    template <class T> void enqueue_stiff(const T *u)
    {
        if (std::is_same<T, float>::value)
            t2_stiff_df_kernel<<<blocks(ntet, 128), 128, 0, stream>>>(ntet, d_shots.as<T2Shot>(), (int)shots.size(),
                                                                      reinterpret_cast<const float *>(u), d_YtK.as<double>());
        else
            t2_stiff_elem_kernel<T><<<blocks(ntet, 128), 128, 0, stream>>>(ntet, d_shots.as<T2Shot>(), (int)shots.size(), u,
                                                                           d_YtK.as<double>());
    }

    // f = K u (element pass + entity pass), u and out device vectors
    template <class T> int enqueue_force(const T *u, T *out)
    {
        enqueue_stiff<T>(u);
        GArgs<T> g = gargs<T>();
        g.Yt = d_YtK.p;
        g.out = out;
        t2_gather_kernel<T, double, G_FORCE, FIN_NONE><<<blocks(nent, 128), 128, 0, stream>>>(nent, d_shots.as<T2Shot>(),
                                                                                             (int)shots.size(), g);
        return 2;
    }

    // x = q(M) b; the last iteration applies FIN with factor h (to U, or to
    // `target` when given); the iterate ends in `xo` (default: the solver's
    // x).  Two forms of an iteration, chosen per handle by timing
    // (choose_iteration): fused, one entity pass that forms the mass rows
    // from the previous iterate and writes the next one to the other of two
    // buffers (the iterates alternate, starting where the last lands in
    // xo); or two-pass, the mass element pass into the per-tetrahedron
    // array, then the entity pass updating x in place.
    // 0: two-pass, 1: fused (one thread per edge or face).  A third form,
    // one thread per node forming all 38 rows from its 18 tetrahedra (each
    // tetrahedron's iterate loaded once, 118 registers), measured 77 us
    // against 68 us (fused) at 48^3 and 30 against 9 us at 16^3; not kept.
    int cheb_form = 0;
    template <class T, int FIN> void launch_fused_iteration(const GArgs<T> &g)
    {
        t2_cheb_kernel<T, FIN><<<blocks(nent, 128), 128, 0, stream>>>(nent, d_shots.as<T2Shot>(), (int)shots.size(), g);
    }
    template <class T, int FIN> int enqueue_solve(const T *b, double h, T *xo = nullptr, T *target = nullptr)
    {
        const int ns = (int)shots.size();
        const bool fused = cheb_form != 0;
        GArgs<T> g = gargs<T>();
        g.b = b;
        g.c0 = cheb_c0;
        g.h = h;
        g.eps = d_eps.as<T>();
        g.Yt = d_YtM.p;
        if (!xo) xo = d_x.as<T>();
        if (target) g.U = target;
        T *buf[2] = {xo, fused ? d_xs.as<T>() : xo};
        int cur = fused ? (mass_iters - 1) % 2 : 0;   // buffer of the first iterate
        g.x = buf[cur];
        if (mass_iters == 1) {
            t2_gather_kernel<T, T, G_CHEB0, FIN><<<blocks(nent, 128), 128, 0, stream>>>(nent, d_shots.as<T2Shot>(), ns, g);
            return 1;
        }
        t2_gather_kernel<T, T, G_CHEB0, FIN_NONE><<<blocks(nent, 128), 128, 0, stream>>>(nent, d_shots.as<T2Shot>(), ns, g);
        int nl = 1;
        for (int k = 1; k < mass_iters; ++k) {
            g.xin = buf[cur];
            cur ^= fused ? 1 : 0;
            g.x = buf[cur];
            g.c1 = cheb_c1[k];
            g.c2 = cheb_c2[k];
            const bool last = k + 1 == mass_iters;
            if (fused) {
                if (last) launch_fused_iteration<T, FIN>(g);
                else launch_fused_iteration<T, FIN_NONE>(g);
                ++nl;
            } else {
                t2_mass_elem_kernel<T><<<blocks(ntet, 128), 128, 0, stream>>>(ntet, d_shots.as<T2Shot>(), ns, d_eps.as<T>(), g.xin,
                                                                              d_YtM.as<T>());
                if (last) t2_gather_kernel<T, T, G_CHEB, FIN><<<blocks(nent, 128), 128, 0, stream>>>(nent, d_shots.as<T2Shot>(), ns, g);
                else t2_gather_kernel<T, T, G_CHEB, FIN_NONE><<<blocks(nent, 128), 128, 0, stream>>>(nent, d_shots.as<T2Shot>(), ns, g);
                nl += 2;
            }
        }
        return nl;
    }

    // Times `n` iterations of the current form in a replayed graph (x, d and
    // b are scratch here); ms per iteration.
    template <class T> double time_iterations(int n)
    {
        const int ns = (int)shots.size();
        GArgs<T> g = gargs<T>();
        g.b = d_b.as<T>();
        g.eps = d_eps.as<T>();
        g.Yt = d_YtM.p;
        g.c1 = 0.5; g.c2 = 0.1;
        T *buf[2] = {d_x.as<T>(), cheb_form ? d_xs.as<T>() : d_x.as<T>()};
        cudaGraph_t gr = nullptr;
        cudaGraphExec_t ex = nullptr;
        EMS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < n; ++k) {
            g.xin = buf[k & 1];
            g.x = buf[(k + 1) & 1];
            if (cheb_form) {
                launch_fused_iteration<T, FIN_NONE>(g);
            } else {
                t2_mass_elem_kernel<T><<<blocks(ntet, 128), 128, 0, stream>>>(ntet, d_shots.as<T2Shot>(), ns, d_eps.as<T>(), g.xin,
                                                                              d_YtM.as<T>());
                t2_gather_kernel<T, T, G_CHEB, FIN_NONE><<<blocks(nent, 128), 128, 0, stream>>>(nent, d_shots.as<T2Shot>(), ns, g);
            }
        }
        cudaError_t ce = cudaStreamEndCapture(stream, &gr);
        if (ce != cudaSuccess) throw Error{EMS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce)};
        ce = cudaGraphInstantiate(&ex, gr, 0);
        if (ce != cudaSuccess) {
            cudaGraphDestroy(gr);
            throw Error{EMS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce)};
        }
        float best = 1e30f;
        for (int r = 0; r < 3; ++r) {   // the first replay warms the caches
            EMS_CUDA(cudaEventRecord(ev0, stream));
            EMS_CUDA(cudaGraphLaunch(ex, stream));
            EMS_CUDA(cudaEventRecord(ev1, stream));
            EMS_CUDA(cudaStreamSynchronize(stream));
            float t = 0;
            EMS_CUDA(cudaEventElapsedTime(&t, ev0, ev1));
            if (r > 0) best = std::min(best, t);
        }
        cudaGraphExecDestroy(ex);
        cudaGraphDestroy(gr);
        return best / n;
    }

    // The faster form of the Chebyshev iteration on this handle's meshes
    // (EMS_TET2_ITERATION=twopass|fused forces one; EMS_TET2_TUNE_LOG prints
    // the times); the forms give the same bits, so the choice changes no result.
    template <class T> void choose_iteration()
    {
        static const char *names[2] = {"twopass", "fused"};
        if (const char *force = std::getenv("EMS_TET2_ITERATION"))
            for (int f = 0; f < 2; ++f)
                if (!std::strcmp(force, names[f])) { cheb_form = f; return; }
        d_x.zero(stream); d_xs.zero(stream); d_d.zero(stream); d_b.zero(stream);
        int best = 0;
        for (int f = 0; f < 2; ++f) {
            cheb_form = f;
            iter_ms[f] = time_iterations<T>(8);
            if (iter_ms[f] < iter_ms[best]) best = f;
        }
        cheb_form = best;
        if (std::getenv("EMS_TET2_TUNE_LOG"))   // diagnostic: the forms' times per iteration
            std::fprintf(stderr, "tet2 iteration (us): twopass %.2f fused %.2f\n", 1e3 * iter_ms[0], 1e3 * iter_ms[1]);
    }
    double iter_ms[2] = {0.0, 0.0};

    double dot_host(const void *x, const void *y)
    {
        if (fp64) t2_dot_kernel<double><<<kDotBlocks, 256, 0, stream>>>(ndof, (const double *)x, (const double *)y, d_part.as<double>());
        else t2_dot_kernel<float><<<kDotBlocks, 256, 0, stream>>>(ndof, (const float *)x, (const float *)y, d_part.as<double>());
        std::vector<double> part(kDotBlocks);
        EMS_CUDA(cudaMemcpyAsync(part.data(), d_part.p, kDotBlocks * 8, cudaMemcpyDeviceToHost, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        double s = 0.0;
        for (double v : part) s += v;
        return s;
    }

    // largest eigenvalue of q(M) K by power iteration with the Rayleigh
    // quotient x.Kx / x.q(M)^-1 x (x = q(M) p)
    template <class T> double lambda_max_t(int iters)
    {
        std::vector<T> x0(ndof, T(0));
        std::vector<unsigned char> live(ndof, 0);
        unsigned long long st = 0x9E3779B97F4A7C15ull;
        for (size_t e = 0; e < ndof; ++e) {
            st ^= st << 13; st ^= st >> 7; st ^= st << 17;
            x0[e] = (T)((double)(st >> 11) / 9007199254740992.0 - 0.5);
        }
        // zero the dead DOFs by one force pass on the start vector's shape: the
        // entity pass writes zeros there; the solve keeps them at zero
        EMS_CUDA(cudaMemcpy(d_x.p, x0.data(), ndof * sizeof(T), cudaMemcpyHostToDevice));
        T *x = d_x.as<T>(), *pb = d_b.as<T>(), *z = d_Uold.as<T>();
        enqueue_force<T>(x, pb);                    // p = K x0
        enqueue_solve<T, FIN_NONE>(pb, 0.0);        // x = q(M) p
        double lam = 0.0;
        for (int it = 0; it < iters; ++it) {
            enqueue_force<T>(x, z);
            const double num = dot_host(x, z), den = dot_host(x, pb);
            lam = num / den;
            EMS_CUDA(cudaMemcpyAsync(pb, z, ndof * sizeof(T), cudaMemcpyDeviceToDevice, stream));
            enqueue_solve<T, FIN_NONE>(pb, 0.0);
            const double nrm = 1.0 / std::sqrt(dot_host(x, x));
            t2_scale_kernel<T><<<blocks(ndof, 256), 256, 0, stream>>>(ndof, x, nrm);
            t2_scale_kernel<T><<<blocks(ndof, 256), 256, 0, stream>>>(ndof, pb, nrm);
        }
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaStreamSynchronize(stream));
        return lam;
    }

    void setup()
    {
        cheb_coefficients();
        if (fp64) launch_pinv_and_eps<double>(); else launch_pinv_and_eps<float>();
        if (fp64) choose_iteration<double>(); else choose_iteration<float>();
        // the power iteration uses the solver's scratch; the state (U, Uold, P) is kept
        DevBuf keep;
        keep.alloc(ndof * (fp64 ? 8 : 4));
        EMS_CUDA(cudaMemcpy(keep.p, d_Uold.p, keep.bytes, cudaMemcpyDeviceToDevice));
        lambda_max = fp64 ? lambda_max_t<double>(100) : lambda_max_t<float>(100);
        EMS_CUDA(cudaMemcpy(d_Uold.p, keep.p, keep.bytes, cudaMemcpyDeviceToDevice));
        dt_lim_n = tet_stability_constant(P.integrator) / std::sqrt(lambda_max);
        dtn = P.dt > 0 ? P.dt / tscale : P.cfl_fraction * dt_lim_n;
        ready = true;
        y_valid = false;
    }

    void locate(const ShotH &S, const double x[3], double val[20][3], size_t dofs[20]) const
    {
        int cell[3];
        double s[3];
        for (int q = 0; q < 3; ++q) {
            int c = (int)std::floor(x[q]);
            c = std::max(0, std::min(c, S.n[q] - 1));
            cell[q] = c;
            s[q] = x[q] - c;
        }
        int ax[3] = {0, 1, 2};   // axes by decreasing fractional coordinate (stable)
        for (int a = 1; a < 3; ++a)
            for (int b = a; b > 0 && s[ax[b - 1]] < s[ax[b]]; --b) std::swap(ax[b], ax[b - 1]);
        int p = 0;
        while (!(kPerm[p][0] == ax[0] && kPerm[p][1] == ax[1] && kPerm[p][2] == ax[2])) ++p;
        const double lam[4] = {1.0 - s[ax[0]], s[ax[0]] - s[ax[1]], s[ax[1]] - s[ax[2]], s[ax[2]]};
        values(p, lam, val);
        const Kuhn k = kuhn(p);
        const Ref &R = ref();
        for (int a = 0; a < 20; ++a) {
            const int *vo = k.vert[R.low[p][a]];
            const size_t node = (size_t)(cell[0] + vo[0]) +
                                (size_t)(S.n[0] + 1) * ((size_t)(cell[1] + vo[1]) + (size_t)(S.n[1] + 1) * (cell[2] + vo[2]));
            dofs[a] = S.dof0 + (size_t)R.plane[p][a] * S.nnode + node;
        }
    }

    bool dead_dof(size_t dof) const
    {
        size_t s = shots.size() - 1;
        while (shots[s].dof0 > dof) --s;
        const ShotH &S = shots[s];
        const size_t l = dof - S.dof0, pl = l / S.nnode, v = l % S.nnode;
        const int et = pl < 14 ? (int)(pl % 7) : 7 + (int)(pl - 14) / 2;
        const int x3[3] = {(int)(v % (S.n[0] + 1)), (int)((v / (S.n[0] + 1)) % (S.n[1] + 1)),
                           (int)(v / ((size_t)(S.n[0] + 1) * (S.n[1] + 1)))};
        const int ax = ref().axes[et];
        for (int q = 0; q < 3; ++q) {
            const int in = (ax >> q) & 1;
            if (x3[q] + in > S.n[q]) return true;
            if (!in && (x3[q] == 0 || x3[q] == S.n[q])) return true;
        }
        return false;
    }

    void add_dipole(int shot, const double pos[3], const double dir[3], int waveform, double f0, double amp)
    {
        EMS_CHECK_ARG(shot >= 0 && shot < (int)shots.size(), "shot index out of range");
        EMS_CHECK_ARG(pos && dir, "position and direction required");
        EMS_CHECK_ARG(waveform == EMS_WAVE_REFERENCE || waveform == EMS_WAVE_RICKER, "unknown waveform");
        EMS_CHECK_ARG(f0 > 0 && std::isfinite(amp), "f0 must be positive");
        const ShotH &S = shots[shot];
        const double xn[3] = {pos[0] / P.h, pos[1] / P.h, pos[2] / P.h};
        for (int q = 0; q < 3; ++q) EMS_CHECK_ARG(xn[q] >= 0 && xn[q] <= S.n[q], "dipole outside the domain");
        EMS_CHECK_ARG(dips.size() < 4096, "at most 4096 dipoles");
        double val[20][3];
        Dip d{};
        locate(S, xn, val, d.dof);
        for (int a = 0; a < 20; ++a)
            d.coef[a] = dead_dof(d.dof[a]) ? 0.0 : (val[a][0] * dir[0] + val[a][1] * dir[1] + val[a][2] * dir[2]) * amp;
        d.kind = waveform;
        d.f0n = f0 * tscale;
        dips.push_back(d);
        rec_nsteps = -1;
    }

    void add_receiver(int shot, const double pos[3])
    {
        EMS_CHECK_ARG(pos != nullptr, "position required");
        EMS_CHECK_ARG(shot >= 0 && shot < (int)shots.size(), "shot index out of range");
        const ShotH &S = shots[shot];
        const double xn[3] = {pos[0] / P.h, pos[1] / P.h, pos[2] / P.h};
        for (int q = 0; q < 3; ++q) EMS_CHECK_ARG(xn[q] >= 0 && xn[q] <= S.n[q], "receiver outside the domain");
        double val[20][3];
        std::array<size_t, 20> d;
        locate(S, xn, val, d.data());
        std::array<double, 60> w;
        for (int a = 0; a < 20; ++a)
            for (int q = 0; q < 3; ++q) w[3 * a + q] = val[a][q];
        rec_dof.push_back(d);
        rec_w.push_back(w);
        rec_nsteps = -1;
    }

    template <class V> void up(DevBuf &b, const std::vector<V> &v)
    {
        b.ensure(std::max<size_t>(v.size(), 1) * sizeof(V));
        if (!v.empty()) EMS_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, stream));
    }

    bool symp() const { return P.integrator != EMS_LEAPFROG; }
    int nsub() const { return P.integrator == EMS_SYMP4 ? 3 : 1; }
    void substeps(double sub[3], double off[3]) const
    {
        const double x1 = 1.0 / (2.0 - std::pow(2.0, 1.0 / 3.0)), x2 = 1.0 - 2.0 * x1;
        sub[0] = dtn; sub[1] = sub[2] = 0.0;
        off[0] = off[1] = off[2] = 0.0;
        if (P.integrator == EMS_SYMP4) {
            sub[0] = x1 * dtn; sub[1] = x2 * dtn; sub[2] = x1 * dtn;
            off[1] = x1 * dtn; off[2] = (x1 + x2) * dtn;
        }
    }

    int nsrc = 0;
    // source table (entries sorted by DOF, in dipole order per DOF), the wave
    // values of every step and substep, receivers and the step counter
    void prepare_run(int nsteps, std::vector<double> &times)
    {
        const int tf = P.time_frequency;
        nobs = (int)rec_dof.size();
        nsamp = nsteps > 0 ? (nsteps - 1) / tf + 1 : 0;
        ncols = 4;
        std::vector<unsigned long long> rd;
        std::vector<double> rw;
        for (int r = 0; r < nobs; ++r) {
            for (int a = 0; a < 20; ++a) rd.push_back(rec_dof[r][a]);
            rw.insert(rw.end(), rec_w[r].begin(), rec_w[r].end());
        }
        up(d_rec_dof, rd);
        up(d_rec_w, rw);
        const size_t ntr = (size_t)std::max(nobs, 1) * std::max(nsamp, 1) * 4;
        d_tr.ensure(ntr * 8);
        d_tr.zero(stream);
        std::vector<std::array<size_t, 2>> ent;   // (dof, dipole * 20 + a)
        for (size_t k = 0; k < dips.size(); ++k)
            for (int a = 0; a < 20; ++a)
                if (dips[k].coef[a] != 0.0) ent.push_back({dips[k].dof[a], 20 * k + a});
        std::stable_sort(ent.begin(), ent.end(), [](const std::array<size_t, 2> &x, const std::array<size_t, 2> &y) { return x[0] < y[0]; });
        std::vector<unsigned long long> sd;
        std::vector<int> sp, sdip;
        std::vector<double> sc;
        for (size_t q = 0; q < ent.size(); ++q) {
            if (q == 0 || ent[q][0] != ent[q - 1][0]) { sd.push_back(ent[q][0]); sp.push_back((int)q); }
            sdip.push_back((int)(ent[q][1] / 20));
            sc.push_back(dips[ent[q][1] / 20].coef[ent[q][1] % 20]);
        }
        sp.push_back((int)ent.size());
        nsrc = (int)sd.size();
        up(d_src_dof, sd);
        up(d_src_ptr, sp);
        up(d_src_dip, sdip);
        up(d_src_coef, sc);
        const size_t nd = std::max<size_t>(dips.size(), 1);
        const int ns = nsub();
        double sub[3], off[3];
        substeps(sub, off);
        std::vector<double> gv((size_t)std::max(nsteps, 1) * ns * nd, 0.0);
        times.assign(std::max(nsamp, 1), 0.0);
        double t = cur_time;
        for (int st = 0; st < nsteps; ++st) {
            for (int q = 0; q < ns; ++q)
                for (size_t k = 0; k < dips.size(); ++k)
                    gv[((size_t)st * ns + q) * nd + k] = tet_wave_value(dips[k].kind, dips[k].f0n, symp() ? t + off[q] + 0.5 * sub[q] : t);
            if (st % tf == 0) times[st / tf] = t;
            t += dtn;
        }
        up(d_src_g, gv);
        EMS_CUDA(cudaMemsetAsync(d_ctl.p, 0, 16, stream));
    }

    size_t snap_bytes() const;
    void save_snapshot(int s);
    void set_checkpoints(int nsnap);
    template <class T> void backward_t(const double *tg, double *grad);
    void backward(const double *tg, size_t ntg, double *grad, size_t ngrad);

    template <class T> int enqueue_step(bool sample = true)
    {
        const int ns = (int)shots.size();
        int nl = 0;
        const int nd = (int)std::max<size_t>(dips.size(), 1);
        if (sample && nobs > 0) {
            t2_sample_kernel<T><<<blocks((unsigned long long)nobs * 32, 128), 128, 0, stream>>>(
                nobs, d_rec_dof.as<unsigned long long>(), d_rec_w.as<double>(), d_U.as<T>(), d_ctl.as<int>(), P.time_frequency,
                nsamp, d_tr.as<double>());
            ++nl;
        }
        if (symp()) {
            double sub[3], off[3];
            substeps(sub, off);
            const int nq = nsub();
            t2_axpy_kernel<T><<<blocks(ndof, 256), 256, 0, stream>>>(ndof, d_U.as<T>(), d_x.as<T>(), 0.5 * sub[0]);
            ++nl;
            for (int q = 0; q < nq; ++q) {
                enqueue_stiff<T>(d_U.as<T>());
                GArgs<T> g = gargs<T>();
                g.Yt = d_YtK.p;
                g.a = sub[q];
                t2_gather_kernel<T, double, G_KICK, FIN_NONE><<<blocks(nent, 128), 128, 0, stream>>>(nent, d_shots.as<T2Shot>(), ns, g);
                nl += 2;
                if (nsrc > 0) {
                    t2_source_kernel<T, 0><<<blocks(nsrc, 128), 128, 0, stream>>>(
                        nsrc, d_src_dof.as<unsigned long long>(), d_src_ptr.as<int>(), d_src_dip.as<int>(), d_src_coef.as<double>(),
                        d_src_g.as<double>(), d_ctl.as<int>(), nq, q, nd, sub[q], d_P.as<double>(), fp64 ? nullptr : d_Pc.as<T>());
                    ++nl;
                }
                const double h = 0.5 * sub[q] + (q + 1 < nq ? 0.5 * sub[q + 1] : 0.0);
                nl += enqueue_solve<T, FIN_DRIFT>(rhs_P<T>(), h);
            }
        } else {
            nl += enqueue_force<T>(d_U.as<T>(), d_b.as<T>());
            if (nsrc > 0) {
                t2_source_kernel<T, 1><<<blocks(nsrc, 128), 128, 0, stream>>>(
                    nsrc, d_src_dof.as<unsigned long long>(), d_src_ptr.as<int>(), d_src_dip.as<int>(), d_src_coef.as<double>(),
                    d_src_g.as<double>(), d_ctl.as<int>(), 1, 0, nd, 1.0, nullptr, d_b.as<T>());
                ++nl;
            }
            nl += enqueue_solve<T, FIN_LEAP>(d_b.as<T>(), dtn * dtn);
        }
        t2_advance_kernel<<<1, 1, 0, stream>>>(d_ctl.as<int>());
        return nl + 1;
    }

    template <class T> void run_t(int nsteps)
    {
        if (!ready) setup();
        rec_nsteps = -1;   // the source table and counters below belong to this run
        std::vector<double> times;
        prepare_run(nsteps, times);
        long long launches = 0;
        if (symp() && !y_valid && nsteps > 0) {   // Y = q(M) P of the current state
            launches += enqueue_solve<T, FIN_NONE>(rhs_P<T>(), 0.0);
            y_valid = true;
        }
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaEventRecord(ev0, stream));
        if (nsteps > 0) {
            struct Graph {
                cudaGraph_t g = nullptr;
                cudaGraphExec_t exec = nullptr;
                ~Graph()
                {
                    if (exec) cudaGraphExecDestroy(exec);
                    if (g) cudaGraphDestroy(g);
                }
            } G;
            EMS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            const int per = enqueue_step<T>();
            cudaError_t ce = cudaStreamEndCapture(stream, &G.g);
            if (ce != cudaSuccess) throw Error{EMS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce)};
            EMS_CUDA(cudaGraphInstantiate(&G.exec, G.g, 0));
            const bool record = ckpt_nsnap > 0 && symp() && cur_time == 0.0 && fresh;
            const int seg = record ? (nsteps + ckpt_nsnap - 1) / ckpt_nsnap : nsteps;
            if (record) d_snap.ensure((size_t)ckpt_nsnap * snap_bytes());
            for (int st = 0; st < nsteps; ++st) {
                if (record && st % seg == 0) save_snapshot(st / seg);
                EMS_CUDA(cudaGraphLaunch(G.exec, stream));
            }
            launches += (long long)per * nsteps;
            if (record) { rec_nsteps = nsteps; rec_seg = seg; }
            else rec_nsteps = -1;
        }
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaEventRecord(ev1, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        float ms = 0;
        EMS_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        last_ms = ms;
        last_launches = launches;
        cur_time += nsteps * dtn;
        fresh = fresh && nsteps == 0;
        const size_t ntr = (size_t)std::max(nobs, 1) * std::max(nsamp, 1) * 4;
        traces.assign(ntr, 0.0);
        EMS_CUDA(cudaMemcpy(traces.data(), d_tr.p, ntr * 8, cudaMemcpyDeviceToHost));
        traces.resize((size_t)nobs * nsamp * 4);
        for (int r = 0; r < nobs; ++r)
            for (int s = 0; s < nsamp; ++s) traces[((size_t)r * nsamp + s) * 4] = times[s] * tscale;
    }

    void run(int nsteps) override
    {
        EMS_CHECK_ARG(nsteps >= 0, "num_steps must be >= 0");
        if (fp64) run_t<double>(nsteps); else run_t<float>(nsteps);
        check_finite({{d_U.p, ndof}}, fp64);
        check_finite({{d_P.p, ndof}}, true);
    }

    size_t field_size(int which) const override
    {
        if (which < 0 || which > 1) throw Error{EMS_ERR_INVALID_ARGUMENT, "field index must be 0 (U) or 1 (P)"};
        return ndof;
    }
    // Fields cross the API node-major (38 * node + plane per shot) and live on
    // the device in planes.  which = 1 is P (symplectic, FP64 on the device)
    // or E^{n-1} (leapfrog).
    void get_field(int which, double *out) const override
    {
        field_size(which);
        std::vector<double> tmp(ndof);
        const bool pfield = which == 1 && symp();
        const DevBuf &b = which == 0 ? d_U : (pfield ? d_P : d_Uold);
        if (pfield || fp64) {
            EMS_CUDA(cudaMemcpy(tmp.data(), b.p, ndof * 8, cudaMemcpyDeviceToHost));
        } else {
            std::vector<float> f(ndof);
            EMS_CUDA(cudaMemcpy(f.data(), b.p, ndof * 4, cudaMemcpyDeviceToHost));
            for (size_t e = 0; e < ndof; ++e) tmp[e] = f[e];
        }
        for (size_t e = 0; e < ndof; ++e) out[e] = tmp[dof_index(e)];
    }
    void set_field(int which, const double *in) override
    {
        field_size(which);
        std::vector<double> tmp(ndof);
        for (size_t e = 0; e < ndof; ++e) tmp[dof_index(e)] = dead_dof(dof_index(e)) ? 0.0 : in[e];
        const bool pfield = which == 1 && symp();
        DevBuf &b = which == 0 ? d_U : (pfield ? d_P : d_Uold);
        if (pfield || fp64) {
            EMS_CUDA(cudaMemcpy(b.p, tmp.data(), ndof * 8, cudaMemcpyHostToDevice));
        } else {
            std::vector<float> f(tmp.begin(), tmp.end());
            EMS_CUDA(cudaMemcpy(b.p, f.data(), ndof * 4, cudaMemcpyHostToDevice));
        }
        if (pfield && !fp64) {
            std::vector<float> f(tmp.begin(), tmp.end());
            EMS_CUDA(cudaMemcpy(d_Pc.p, f.data(), ndof * 4, cudaMemcpyHostToDevice));
        }
        y_valid = false;
        fresh = false;
        rec_nsteps = -1;
    }

    void save(const char *path) const override
    {
        EMS_CHECK_ARG(path && *path, "file name required");
        for (int o = 0; o < nobs; ++o) {
            std::string fn = path;
            if (o > 0) {
                size_t dot = fn.rfind('.');
                std::string suf = "_" + std::to_string(o);
                if (dot == std::string::npos) fn += suf; else fn.insert(dot, suf);
            }
            std::ofstream f(fn);
            if (!f.is_open()) throw Error{EMS_ERR_IO, "cannot open " + fn};
            f << std::setprecision(15) << std::scientific << "time,Ex,Ey,Ez" << std::endl;
            for (int s = 0; s < nsamp; ++s) {
                const double *r = &traces[((size_t)o * nsamp + s) * 4];
                f << r[0] << "," << r[1] << "," << r[2] << "," << r[3] << std::endl;
            }
        }
    }

    bool fresh = true;   // the state is the reset state (zero fields at t = 0)
    void reset() override
    {
        d_U.zero(stream); d_Uold.zero(stream); d_P.zero(stream); d_x.zero(stream); d_xs.zero(stream); d_d.zero(stream);
        d_b.zero(stream);
        if (d_Pc.p) d_Pc.zero(stream);
        cur_time = 0.0;
        fresh = true;
        y_valid = false;
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    void launch_shape(int b[3]) override { b[0] = 128; b[1] = b[2] = 1; }

    // One Chebyshev iteration in the handle's form replayed in a graph of
    // `launches` iterations; bytes: x (read and written), b, d (read and
    // written), the block inverses and eps once per iteration (a fused
    // iteration's minimum: the neighbours' x re-read by the mass rows hit the
    // caches; the two-pass form also moves the per-tetrahedron array).
    void time_dominant(int launches, double *ms, double *bytes, std::string *name) override
    {
        if (!ready) setup();
        d_x.zero(stream); d_xs.zero(stream); d_d.zero(stream); d_b.zero(stream);
        *ms = fp64 ? time_iterations<double>(std::max(launches, 1)) : time_iterations<float>(std::max(launches, 1));
        *bytes = (double)(fp64 ? 8 : 4) * (5.0 * ndof + ntet + 3.0 * nent);
        y_valid = false;
        static const char *kern[2] = {"t2_mass_elem_kernel + t2_gather_kernel<", "t2_cheb_kernel<"};
        *name = std::string(kern[cheb_form]) + (fp64 ? "double>" : "float>");
    }

    // f = K u in the handle's precision (API DOF order)
    void apply_stiffness(const double *u, double *f)
    {
        std::vector<double> tmp(ndof);
        for (size_t e = 0; e < ndof; ++e) tmp[dof_index(e)] = u[e];
        auto body = [&](auto tag) {
            using T = decltype(tag);
            std::vector<T> in(tmp.begin(), tmp.end()), out(ndof);
            DevBuf a, b;
            a.alloc(ndof * sizeof(T));
            b.alloc(ndof * sizeof(T));
            EMS_CUDA(cudaMemcpy(a.p, in.data(), ndof * sizeof(T), cudaMemcpyHostToDevice));
            enqueue_force<T>(a.as<T>(), b.as<T>());
            EMS_CUDA(cudaGetLastError());
            EMS_CUDA(cudaStreamSynchronize(stream));
            EMS_CUDA(cudaMemcpy(out.data(), b.p, ndof * sizeof(T), cudaMemcpyDeviceToHost));
            for (size_t e = 0; e < ndof; ++e) f[e] = (double)out[dof_index(e)];
        };
        if (fp64) body(double()); else body(float());
    }

    // H = 1/2 P.q(M)P + 1/2 U.KU in FP64 (symplectic state)
    void energy(double *out, int n)
    {
        EMS_CHECK_ARG(symp(), "energy is defined for the symplectic integrators");
        EMS_CHECK_ARG(out && n == (int)shots.size(), "one value per shot");
        if (!ready) setup();
        std::vector<double> U(ndof), Pv(ndof);
        get_field(0, U.data());
        get_field(1, Pv.data());
        // an FP64 twin of this handle computes the products
        ems_tetfem_params p2 = P;
        p2.precision = EMS_FP64;
        p2.dt = dtn * tscale;
        std::vector<std::array<int, 3>> cells;
        for (auto &s : shots) cells.push_back({s.n[0], s.n[1], s.n[2]});
        Tet2Sim tw(&p2, cells);
        tw.eps_h = eps_h;
        tw.cheb_coefficients();
        tw.launch_pinv_and_eps<double>();
        tw.set_field(0, U.data());
        tw.set_field(1, Pv.data());
        tw.enqueue_force<double>(tw.d_U.as<double>(), tw.d_b.as<double>());        // b = K U
        tw.enqueue_solve<double, FIN_NONE>(tw.d_P.as<double>(), 0.0);              // x = q(M) P
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaStreamSynchronize(tw.stream));
        std::vector<double> KU(ndof), Y(ndof), Ud(ndof), Pd(ndof);
        EMS_CUDA(cudaMemcpy(KU.data(), tw.d_b.p, ndof * 8, cudaMemcpyDeviceToHost));
        EMS_CUDA(cudaMemcpy(Y.data(), tw.d_x.p, ndof * 8, cudaMemcpyDeviceToHost));
        EMS_CUDA(cudaMemcpy(Ud.data(), tw.d_U.p, ndof * 8, cudaMemcpyDeviceToHost));
        EMS_CUDA(cudaMemcpy(Pd.data(), tw.d_P.p, ndof * 8, cudaMemcpyDeviceToHost));
        for (size_t s = 0; s < shots.size(); ++s) {
            double e = 0.0;
            const size_t a = shots[s].dof0, b = a + kPlanes * shots[s].nnode;
            for (size_t q = a; q < b; ++q) e += 0.5 * (Pd[q] * Y[q] + Ud[q] * KU[q]);
            out[s] = e;
        }
    }
};

// ---------------------------------------------------------------- adjoint
// Reverse sweep of a recorded symplectic run (zero start state):
//   forward step n (merged drifts): U += a_0/2 Y_0; for each substage q:
//     P -= a_q (K U - f), Y_{q+1} = q(M) P, U += h_q Y_{q+1}
//   reversed: for q = last..0: Z = q(M) Ubar, Pbar += h_q Z,
//     grad -= h_q Z . dM/deps Y_{q+1}, Ubar -= a_q K Pbar; then the start
//     drift (a_0/2, Y_0) and the receiver samples of step n (Ubar += w g).
// dY/deps is taken as the derivative of M^-1 P (-q(M) M_t Y), within the
// polynomial's error of the derivative of q(M) P.  Each segment between
// snapshots is recomputed once, keeping (U, P) of its steps; each reversed
// step recomputes its drift increments Y_0..Y_nsub from (U_n, P_n).  Ubar
// accumulates the stiffness terms in FP64 (as P does forward) with a copy
// in the run precision for the solves; Pbar is in the run precision.
size_t Tet2Sim::snap_bytes() const { return ndof * ((fp64 ? 8 : 4) + 8); }

void Tet2Sim::save_snapshot(int s)
{
    char *b = d_snap.as<char>() + (size_t)s * snap_bytes();
    const size_t w = ndof * (fp64 ? 8 : 4);
    EMS_CUDA(cudaMemcpyAsync(b, d_U.p, w, cudaMemcpyDeviceToDevice, stream));
    EMS_CUDA(cudaMemcpyAsync(b + w, d_P.p, ndof * 8, cudaMemcpyDeviceToDevice, stream));
}

void Tet2Sim::set_checkpoints(int nsnap)
{
    EMS_CHECK_ARG(nsnap >= 0, "nsnap must be >= 0");
    if (!symp()) throw Error{EMS_ERR_UNSUPPORTED, "the adjoint needs a symplectic integrator"};
    ckpt_nsnap = nsnap;
    rec_nsteps = -1;
    if (nsnap == 0) d_snap.release();
}

template <class T> void Tet2Sim::backward_t(const double *tg, double *grad)
{
    const int ns = (int)shots.size(), nq = nsub();
    const int nsteps = rec_nsteps, seg = rec_seg;
    const size_t w = ndof * sizeof(T);
    double sub[3], off[3];
    substeps(sub, off);
    double hq[3];
    for (int k = 0; k < nq; ++k) hq[k] = 0.5 * sub[k] + (k + 1 < nq ? 0.5 * sub[k + 1] : 0.0);
    // receiver adjoint loads: entries by DOF, table per step (zero off the sampling steps)
    const int tf = P.time_frequency;
    std::vector<std::array<size_t, 2>> ent;   // (dof, (r * 3 + c) * 20 + a)
    for (int r = 0; r < nobs; ++r)
        for (int a = 0; a < 20; ++a)
            for (int c = 0; c < 3; ++c)
                if (rec_w[r][3 * a + c] != 0.0 && !dead_dof(rec_dof[r][a])) ent.push_back({rec_dof[r][a], (size_t)(r * 3 + c) * 20 + a});
    std::stable_sort(ent.begin(), ent.end(), [](const std::array<size_t, 2> &x, const std::array<size_t, 2> &y) { return x[0] < y[0]; });
    std::vector<unsigned long long> rd;
    std::vector<int> rp, ri;
    std::vector<double> rc;
    for (size_t q = 0; q < ent.size(); ++q) {
        if (q == 0 || ent[q][0] != ent[q - 1][0]) { rd.push_back(ent[q][0]); rp.push_back((int)q); }
        const size_t rcid = ent[q][1] / 20, a = ent[q][1] % 20;
        ri.push_back((int)rcid);
        rc.push_back(rec_w[rcid / 3][3 * a + rcid % 3]);
    }
    rp.push_back((int)ent.size());
    const int nrd = (int)rd.size(), nd3 = std::max(3 * nobs, 1);
    std::vector<double> gt((size_t)nsteps * nd3, 0.0);
    for (int n = 0; n < nsteps; n += tf)
        for (int r = 0; r < nobs; ++r)
            for (int c = 0; c < 3; ++c) gt[(size_t)n * nd3 + 3 * r + c] = tg[((size_t)r * nsamp + n / tf) * 4 + 1 + c];
    DevBuf a_dof, a_ptr, a_idx, a_coef, a_g;
    up(a_dof, rd); up(a_ptr, rp); up(a_idx, ri); up(a_coef, rc); up(a_g, gt);
    // buffers: the drift increments of the segment's steps, adjoint state,
    // gradient, end state.  Increment q of step n (q(M) P before the first
    // drift, q = 0, and after kick q, q = 1..nq) sits in slot n * nq + q of
    // the segment, so the last one of step n is the first of step n + 1 (the
    // same P); the recompute keeps them and the reversed steps read them.
    DevBuf Ys, Ub, Ubc, Pb, gd, keepU, keepP;
    Ys.alloc(((size_t)seg * nq + 1) * w);
    Ub.alloc(ndof * 8);
    Pb.alloc(w);
    if (!fp64) Ubc.alloc(w);
    gd.alloc(ntet * 8);
    keepU.alloc(w);
    keepP.alloc(ndof * 8);
    EMS_CUDA(cudaMemcpyAsync(keepU.p, d_U.p, w, cudaMemcpyDeviceToDevice, stream));
    EMS_CUDA(cudaMemcpyAsync(keepP.p, d_P.p, ndof * 8, cudaMemcpyDeviceToDevice, stream));
    Ub.zero(stream); Pb.zero(stream); gd.zero(stream);
    if (Ubc.p) Ubc.zero(stream);
    T *Ubr = fp64 ? Ub.as<T>() : Ubc.as<T>();   // Ubar in the run precision (right-hand side of the solves)
    int nseg0 = 0;   // first step of the segment being reversed
    auto Y = [&](int n, int q) { return Ys.as<T>() + ((size_t)(n - nseg0) * nq + q) * ndof; };
    const int nd = (int)std::max<size_t>(dips.size(), 1);
    int *ctl = d_ctl.as<int>();
    auto narrowP = [&]() {
        if (!fp64) t2_narrow_kernel<T><<<blocks(ndof, 256), 256, 0, stream>>>(ndof, d_P.as<double>(), d_Pc.as<T>());
    };
    for (int s = (nsteps - 1) / seg; s >= 0; --s) {
        const int n0 = s * seg, n1 = std::min(nsteps, n0 + seg);
        nseg0 = n0;
        // recompute the segment from its snapshot (the forward step's
        // kernels and arithmetic: the half drift with the previous step's
        // last increment, then per substep stiffness, kick, source and the
        // solve whose drift ends the substep), keeping the increments
        const char *sb = d_snap.as<char>() + (size_t)s * snap_bytes();
        EMS_CUDA(cudaMemcpyAsync(d_U.p, sb, w, cudaMemcpyDeviceToDevice, stream));
        EMS_CUDA(cudaMemcpyAsync(d_P.p, sb + w, ndof * 8, cudaMemcpyDeviceToDevice, stream));
        narrowP();
        enqueue_solve<T, FIN_NONE>(rhs_P<T>(), 0.0, Y(n0, 0));
        t2_set_kernel<<<1, 1, 0, stream>>>(ctl, n0);
        for (int n = n0; n < n1; ++n) {
            t2_axpy_kernel<T><<<blocks(ndof, 256), 256, 0, stream>>>(ndof, d_U.as<T>(), Y(n, 0), 0.5 * sub[0]);
            for (int q = 0; q < nq; ++q) {
                enqueue_stiff<T>(d_U.as<T>());
                GArgs<T> g = gargs<T>();
                g.Yt = d_YtK.p;
                g.a = sub[q];
                t2_gather_kernel<T, double, G_KICK, FIN_NONE><<<blocks(nent, 128), 128, 0, stream>>>(nent, d_shots.as<T2Shot>(), ns, g);
                if (nsrc > 0)
                    t2_source_kernel<T, 0><<<blocks(nsrc, 128), 128, 0, stream>>>(
                        nsrc, d_src_dof.as<unsigned long long>(), d_src_ptr.as<int>(), d_src_dip.as<int>(), d_src_coef.as<double>(),
                        d_src_g.as<double>(), ctl, nq, q, nd, sub[q], d_P.as<double>(), fp64 ? nullptr : d_Pc.as<T>());
                enqueue_solve<T, FIN_DRIFT>(rhs_P<T>(), hq[q], Y(n, q + 1));
            }
            t2_advance_kernel<<<1, 1, 0, stream>>>(ctl);
        }
        // reversed steps
        for (int n = n1 - 1; n >= n0; --n) {
            t2_set_kernel<<<1, 1, 0, stream>>>(ctl, n);
            // adjoint of the substages
            for (int q = nq - 1; q >= 0; --q) {
                enqueue_solve<T, FIN_DRIFT>(Ubr, hq[q], d_x.as<T>(), Pb.as<T>());
                t2_grad_kernel<T><<<blocks(ntet, 128), 128, 0, stream>>>(ntet, d_shots.as<T2Shot>(), ns, d_x.as<T>(), Y(n, q + 1),
                                                                         -hq[q], gd.as<double>());
                enqueue_stiff<T>(Pb.as<T>());
                GArgs<T> g = gargs<T>();
                g.Yt = d_YtK.p;
                g.a = sub[q];
                g.P = Ub.as<double>();
                g.Pc = fp64 ? nullptr : Ubc.as<T>();
                t2_gather_kernel<T, double, G_KICK, FIN_NONE><<<blocks(nent, 128), 128, 0, stream>>>(nent, d_shots.as<T2Shot>(), ns, g);
            }
            enqueue_solve<T, FIN_DRIFT>(Ubr, 0.5 * sub[0], d_x.as<T>(), Pb.as<T>());
            t2_grad_kernel<T><<<blocks(ntet, 128), 128, 0, stream>>>(ntet, d_shots.as<T2Shot>(), ns, d_x.as<T>(), Y(n, 0),
                                                                     -0.5 * sub[0], gd.as<double>());
            if (nrd > 0 && n % tf == 0)
                t2_source_kernel<T, 0><<<blocks(nrd, 128), 128, 0, stream>>>(
                    nrd, a_dof.as<unsigned long long>(), a_ptr.as<int>(), a_idx.as<int>(), a_coef.as<double>(), a_g.as<double>(),
                    ctl, 1, 0, nd3, 1.0, Ub.as<double>(), fp64 ? nullptr : Ubc.as<T>());
            EMS_CUDA(cudaGetLastError());
        }
    }
    EMS_CUDA(cudaMemcpyAsync(d_U.p, keepU.p, w, cudaMemcpyDeviceToDevice, stream));
    EMS_CUDA(cudaMemcpyAsync(d_P.p, keepP.p, ndof * 8, cudaMemcpyDeviceToDevice, stream));
    narrowP();
    y_valid = false;
    std::vector<double> g(ntet);
    EMS_CUDA(cudaStreamSynchronize(stream));
    EMS_CUDA(cudaMemcpy(g.data(), gd.p, ntet * 8, cudaMemcpyDeviceToHost));
    // dJ/deps_r: the mass scales with eps_r; back to the API order
    for (size_t t = 0; t < ntet; ++t) grad[t] = g[tet_index(t)];
}

void Tet2Sim::backward(const double *tg, size_t ntg, double *grad, size_t ngrad)
{
    EMS_CHECK_ARG(tg && grad, "trace gradient and output required");
    EMS_CHECK_ARG(ngrad == ntet, "gradient must have one value per tetrahedron");
    if (rec_nsteps < 0 || d_snap.p == nullptr) throw Error{EMS_ERR_STATE, "no recorded run: set checkpoints, reset and run first"};
    EMS_CHECK_ARG(ntg == (size_t)nobs * nsamp * 4, "trace gradient must have the shape of the traces");
    if (fp64) backward_t<double>(tg, grad); else backward_t<float>(tg, grad);
    for (size_t t = 0; t < ntet; ++t)
        if (!std::isfinite(grad[t])) throw Error{EMS_ERR_NOT_FINITE, "the gradient holds a NaN or an Inf"};
}

bool is_tet2(const Sim *s) { return dynamic_cast<const Tet2Sim *>(s) != nullptr; }

Sim *make_tet2(const ems_tetfem_params *p, const std::vector<std::array<int, 3>> &cells) { return new Tet2Sim(p, cells); }

void tet2_set_material(Sim *s, const double *eps_r, const double *sigma) { static_cast<Tet2Sim *>(s)->set_material(eps_r, sigma); }
void tet2_add_dipole(Sim *s, int shot, const double pos[3], const double dir[3], int waveform, double f0, double amp)
{
    static_cast<Tet2Sim *>(s)->add_dipole(shot, pos, dir, waveform, f0, amp);
}
void tet2_add_receiver(Sim *s, int shot, const double pos[3]) { static_cast<Tet2Sim *>(s)->add_receiver(shot, pos); }
void tet2_time_step(const Sim *s, double *dt, double *lim)
{
    auto *f = const_cast<Tet2Sim *>(static_cast<const Tet2Sim *>(s));
    if (!f->ready) f->setup();
    if (dt) *dt = f->dtn * f->tscale;
    if (lim) *lim = f->dt_lim_n * f->tscale;
}
void tet2_apply_stiffness(Sim *s, const double *u, double *f, size_t n)
{
    auto *t = static_cast<Tet2Sim *>(s);
    EMS_CHECK_ARG(u && f, "input and output required");
    EMS_CHECK_ARG(n == t->ndof, "vector length must be 38*(nx+1)*(ny+1)*(nz+1) per shot");
    t->apply_stiffness(u, f);
}
void tet2_energy(Sim *s, double *out, int n) { static_cast<Tet2Sim *>(s)->energy(out, n); }
void tet2_set_checkpoints(Sim *s, int nsnap) { static_cast<Tet2Sim *>(s)->set_checkpoints(nsnap); }
void tet2_backward(Sim *s, const double *trace_grad, size_t ntg, double *grad_eps, double *grad_sigma, size_t ngrad)
{
    if (grad_sigma) throw Error{EMS_ERR_UNSUPPORTED, "order-2 tetrahedra have no conductivity gradient"};
    static_cast<Tet2Sim *>(s)->backward(trace_grad, ntg, grad_eps, ngrad);
}
size_t tet2_ntet(const Sim *s) { return static_cast<const Tet2Sim *>(s)->ntet; }

// Reference matrices of the second-order element as the solver computes them.
void tet2_element_matrices(int type, double *M, double *K)
{
    EMS_CHECK_ARG(type >= 0 && type < 6, "tetrahedron type must be 0..5");
    const Ref &R = ref();
    std::copy(R.M[type], R.M[type] + 400, M);
    std::copy(R.K[type], R.K[type] + 400, K);
}

}  // namespace ems
