// Tetrahedral edge-element (Whitney / lowest-order Nedelec) FEM on one GPU.
//
// The reference has hexahedral elements only; this solver carries its
// symplectic and leapfrog time loops (symplectic_2/fem_simulation.cpp:557-672,
// symplectic_4/fem_simulation.cpp:1347-1350, fem_v2/fem_simulation.cpp:
// 627-654) to a mesh of cubes split into six Kuhn tetrahedra:
//
//   DOF names    edge slot e = 7*node + d, d over the 7 edge directions
//                leaving a node (mesh tables, flags, the API).
//   layout       the time loop's arrays in planes: slot d of node v at
//                d*nnode + v (fslot); packed mass blocks in seven vec4 planes.
//   time step    tet_step_kernel, one thread per node and one launch per
//                substep: the curls of the node's 18 tetrahedra recomputed
//                from the 43 edge values around it (no per-tetrahedron array
//                in the loop), the curl-transpose summed over them in
//                ascending tetrahedron order (deterministic, no atomics), the
//                kick, the mass-block drift; U alternates between two
//                buffers.  The receivers are sampled by leading blocks of a
//                step's first launch.
//   mass inverse per-node 7x7 blocks, built and inverted in FP64 on the GPU
//                (tet_minv_setup_kernel), stored packed symmetric in the run
//                precision; applied inside tet_step_kernel from registers.
//   adjoint      the same kernel runs the reversed steps (see "adjoint").
//   FP32 runs    the symplectic kick in double-float arithmetic: the
//                gathered force as hi + lo, the increment split exactly, P
//                with a bfloat16 compensation plane (see "compensated
//                updates").
// Units are normalised (cube edge 1, c0 = 1); the API converts.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <unordered_map>
#include <utility>

#include "ems_internal.hpp"

namespace ems {

namespace {

const int kPerm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
const int kLoc[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
const int kDir[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
// Per-slot flag byte: the slot is PEC or unused (no DOF), or it carries a
// dipole load (only those slots search the source list).
constexpr unsigned char kPecBit = 1, kSrcBit = 2, kRecBit = 4;   // kRecBit: a receiver reads the slot
constexpr double kEps0 = 8.8541878128e-12;   // vacuum permittivity, F/m

struct Shape {
    double grad[4][3];
    int vert[4][3];
    double curl[6][3], wint[6][3], wsq[6];
};

Shape make_shape(int p)
{
    Shape s{};
    int a = kPerm[p][0], b = kPerm[p][1], c = kPerm[p][2];
    s.grad[0][a] = -1.0;
    s.grad[1][a] = 1.0; s.grad[1][b] = -1.0;
    s.grad[2][b] = 1.0; s.grad[2][c] = -1.0;
    s.grad[3][c] = 1.0;
    s.vert[1][a] = 1;
    s.vert[2][a] = 1; s.vert[2][b] = 1;
    s.vert[3][0] = s.vert[3][1] = s.vert[3][2] = 1;
    const double vol = 1.0 / 6.0;
    for (int l = 0; l < 6; ++l) {
        const double *gm = s.grad[kLoc[l][0]], *gn = s.grad[kLoc[l][1]];
        s.curl[l][0] = 2.0 * (gm[1] * gn[2] - gm[2] * gn[1]);
        s.curl[l][1] = 2.0 * (gm[2] * gn[0] - gm[0] * gn[2]);
        s.curl[l][2] = 2.0 * (gm[0] * gn[1] - gm[1] * gn[0]);
        for (int q = 0; q < 3; ++q) s.wint[l][q] = vol / 4.0 * (gn[q] - gm[q]);
        double nn = gn[0] * gn[0] + gn[1] * gn[1] + gn[2] * gn[2];
        double mm = gm[0] * gm[0] + gm[1] * gm[1] + gm[2] * gm[2];
        double mn = gm[0] * gn[0] + gm[1] * gn[1] + gm[2] * gn[2];
        s.wsq[l] = vol / 10.0 * (nn - mn + mm);
    }
    return s;
}

int dir_index(int dx, int dy, int dz)
{
    for (int d = 0; d < 7; ++d)
        if (kDir[d][0] == dx && kDir[d][1] == dy && kDir[d][2] == dz) return d;
    return -1;
}

}  // namespace

// Shape tables in constant memory: curl of the six Whitney functions of each
// of the six Kuhn tetrahedron types (scaled by nothing: unit cube).
__constant__ double c_wint[6][6][3];
__constant__ double c_wsq[6][6];
__constant__ int c_dir[7][3];
__constant__ unsigned char c_pack[7][7];   // packed symmetric index of (r,c)


// ---------------------------------------------------------------- setup
__device__ void sym3_eig(double A[3][3], double w[3], double V[3][3])
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) V[i][j] = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
        // converged: the off-diagonal sum at the rounding floor (exact zero
        // is rarely reached, and each further sweep only rounds again)
        if (off <= 1e-14 * (fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]))) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (A[p][q] == 0.0) continue;
                double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {
                    double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - s * akq;
                    A[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - s * aqk;
                    A[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < 3; ++i) w[i] = A[i][i];
}

__device__ void sym3_pinv(const double Ain[3][3], double P[3][3])
{
    double A[3][3], w[3], V[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = Ain[i][j];
    sym3_eig(A, w, V);
    double mx = fmax(fabs(w[0]), fmax(fabs(w[1]), fabs(w[2])));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
                if (w[k] > 1e-10 * mx) s += V[i][k] * V[j][k] / w[k];
            P[i][j] = s;
        }
}

// Plane layout of the time loop's arrays: slot d of node v (edge slot
// e = 7 v + d of the mesh tables, the flags and the API) at d * nnode + v,
// so a warp of consecutive nodes reads and writes contiguous memory for
// every slot; the packed symmetric mass block of node v (28 entries) as
// seven planes of four, entry p at ((p / 4) * nnode + v) * 4 + p % 4.
__host__ __device__ __forceinline__ size_t fslot(size_t e, size_t nnode) { return (e % 7) * nnode + e / 7; }
__host__ __device__ __forceinline__ size_t fpk(size_t v, int p, size_t nnode)
{
    return ((size_t)(p >> 2) * nnode + v) * 4 + (p & 3);
}

// Per-node inverse mass block in FP64: M_v = W S^+ W^T + alpha (I - D G^+ D^T)
// over the node's active slots (W_i = sum_T eps_T int_T w_i, D_i the edge
// vector, S = sym(D^T W), G = D^T D, alpha = mean consistent diagonal), then
// inverted by Cholesky.  Writes the packed block (28 entries) in the plane
// layout in FP64 and, when pk32 is given, in FP32; *status = 1 if a block
// is not positive definite.
__global__ void __launch_bounds__(128) tet_minv_setup_kernel(size_t nnode, const unsigned char *__restrict__ pec,
                                                             const int *__restrict__ inc_ptr, const int *__restrict__ inc,
                                                             const double *__restrict__ eps, double *__restrict__ pk64,
                                                             float *__restrict__ pk32, int *__restrict__ status)
{
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nnode) return;
    // entry (i, j), j >= i, of the packed block in the plane layout, FP64
    // and (for FP32 runs) FP32
    auto put = [&](int i, int j, double x) {
        const size_t f = fpk(v, i * (13 - i) / 2 + j, nnode);
        pk64[f] = x;
        if (pk32) pk32[f] = (float)x;
    };
    // Slots are indexed by their direction d, a compile-time index once the
    // loops are unrolled, so every array below stays in registers.  A PEC or
    // unused slot enters the block as an identity row and column: the
    // factors of the active slots gain only exact-zero terms, and its row
    // and column of the inverse are written as zeros.
    bool live[7];
    int k = 0;
    double W[7][3], diag[7];
#pragma unroll
    for (int d = 0; d < 7; ++d) {
        const size_t e = 7 * v + d;
        live[d] = !(pec[e] & kPecBit);
        k += live[d] ? 1 : 0;
        W[d][0] = W[d][1] = W[d][2] = 0.0;
        diag[d] = 0.0;
        if (live[d])
            for (int s = inc_ptr[e]; s < inc_ptr[e + 1]; ++s) {
                const int t = inc[s] >> 3, l = inc[s] & 7, p = t % 6;
                const double ep = eps[t];
#pragma unroll
                for (int q = 0; q < 3; ++q) W[d][q] += ep * c_wint[p][l][q];
                diag[d] += ep * c_wsq[p][l];
            }
    }
    if (k == 0) {
#pragma unroll
        for (int i = 0; i < 7; ++i)
#pragma unroll
            for (int j = i; j < 7; ++j) put(i, j, 0.0);
        return;
    }
    double S[3][3], G[3][3], Sp[3][3], Gp[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            double s1 = 0.0, s2 = 0.0, g = 0.0;
#pragma unroll
            for (int d = 0; d < 7; ++d)
                if (live[d]) {
                    s1 += c_dir[d][a] * W[d][b];
                    s2 += W[d][a] * c_dir[d][b];
                    g += c_dir[d][a] * c_dir[d][b];
                }
            S[a][b] = 0.5 * (s1 + s2);
            G[a][b] = g;
        }
    sym3_pinv(S, Sp);
    sym3_pinv(G, Gp);
    double alpha = 0.0;
#pragma unroll
    for (int d = 0; d < 7; ++d)
        if (live[d]) alpha += diag[d];
    alpha /= k;
    // lower triangle, packed by rows: entry (i, j), j <= i, at i (i + 1) / 2 + j
    double A[28];
#pragma unroll
    for (int i = 0; i < 7; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            double m = i == j ? 1.0 : 0.0;
            if (live[i] && live[j]) {
                double ws = 0.0, dq = 0.0;
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = 0; b < 3; ++b) {
                        ws += W[i][a] * Sp[a][b] * W[j][b];
                        dq += c_dir[i][a] * Gp[a][b] * c_dir[j][b];
                    }
                m = ws + alpha * ((i == j ? 1.0 : 0.0) - dq);
            }
            A[i * (i + 1) / 2 + j] = m;
        }
    // Cholesky factor L in place
#pragma unroll
    for (int i = 0; i < 7; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            double s = A[i * (i + 1) / 2 + j];
#pragma unroll
            for (int q = 0; q < j; ++q) s -= A[i * (i + 1) / 2 + q] * A[j * (j + 1) / 2 + q];
            if (i == j) {
                if (!(s > 0.0)) {
                    *status = 1;
                    return;
                }
                A[i * (i + 1) / 2 + i] = sqrt(s);
            } else {
                A[i * (i + 1) / 2 + j] = s / A[j * (j + 1) / 2 + j];
            }
        }
    // L^-1 in place, row by row (row i reads its own L entries at q >= j,
    // not yet overwritten, and the inverted rows above it)
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        const double lii = A[i * (i + 1) / 2 + i];
#pragma unroll
        for (int j = 0; j < i; ++j) {
            double s = 0.0;
#pragma unroll
            for (int q = j; q < i; ++q) s += A[i * (i + 1) / 2 + q] * A[q * (q + 1) / 2 + j];
            A[i * (i + 1) / 2 + j] = -s / lii;
        }
        A[i * (i + 1) / 2 + i] = 1.0 / lii;
    }
    // Minv = L^-T L^-1
#pragma unroll
    for (int i = 0; i < 7; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            double s = 0.0;
#pragma unroll
            for (int q = i; q < 7; ++q) s += A[q * (q + 1) / 2 + i] * A[q * (q + 1) / 2 + j];
            put(j, i, live[i] && live[j] ? s : 0.0);
        }
}


// ---------------------------------------------------------------- time step
template <class T> struct alignas(4 * sizeof(T)) vec4 {
    T x, y, z, w;
};

// packed upper-triangle index of (r, c) in a symmetric 7x7 block
__device__ __forceinline__ int pk7(int r, int c)
{
    int a = r < c ? r : c, b = r < c ? c : r;
    return a * (13 - a) / 2 + b;
}

// The packed mass block of node v (plane layout) into registers.
template <class T> __device__ __forceinline__ void load_block(const T *__restrict__ minv, size_t nnode, size_t v, T (&mv)[28])
{
    const vec4<T> *m4 = reinterpret_cast<const vec4<T> *>(minv);
#pragma unroll
    for (int q = 0; q < 7; ++q) {
        const vec4<T> w = m4[(size_t)q * nnode + v];
        mv[4 * q] = w.x; mv[4 * q + 1] = w.y; mv[4 * q + 2] = w.z; mv[4 * q + 3] = w.w;
    }
}

// (Minv_v x)_d from the packed block, terms in j order.
template <class T> __device__ __forceinline__ T block_row(const T (&mv)[28], const T (&x)[7], int d)
{
    T y = 0;
#pragma unroll
    for (int j = 0; j < 7; ++j) {
        const int r7 = d < j ? d : j, s7 = d < j ? j : d;
        y = fma(mv[r7 * (13 - r7) / 2 + s7], x[j], y);
    }
    return y;
}

// ------------------------------------------------ compensated updates
// K has a large null space (discrete gradients), and a force K U rounded
// to FP32 has a small component in it.  Nothing restores the field there:
// that rounding noise random-walks in P and its integral grows in U roughly
// as t^1.5, so the FP32-vs-FP64 trace error grew faster than linearly with
// the run length (1.1e-4 of the field after 2000 steps on a 32^3 mesh,
// 1.5e-4 after 4000 on 48^3).  Compensating only the sums P + increment and
// U + increment did not change that.  FP32 runs therefore evaluate the
// kick in double-float arithmetic: the gathered force is kept as hi + lo
// (each curl term is an exact product, added by an error-free two-sum,
// Knuth), the increment a (f_hi + f_lo) is split exactly with one fused
// multiply-add, and P carries its own rounding error in a bfloat16 plane
// (true value ~ hi + lo, |lo| <= ulp(hi)/2) that enters the next kick of
// that slot.  Only hi enters Minv P; lo is node-local and updated in place.
// Curl rounding needs no care: it perturbs B, and K's image of any B stays
// outside the null space.  The drift's rounding needs none either: an
// emulation of the 32^3 headline run (2000 steps, FP64 reference) gave
// 5.9e-6 with U compensated as well and 5.7e-6 without, against 1.3e-4
// for plain FP32 and 2.9e-5 when the gathered force is rounded once.
struct Comp {
    __nv_bfloat16 *p = nullptr;   // compensation of P (the field the kick updates)
};

// s = a + b rounded, err = (a + b) - s exactly (six flops, no ordering
// assumption on |a|, |b|; no multiplications, so nothing is contracted).
template <class T> __device__ __forceinline__ T two_sum(T a, T b, T &err)
{
    const T s = a + b;
    const T bb = s - a;
    err = (a - (s - bb)) + (b - bb);
    return s;
}

// A rounded product that the compiler may not fuse into a following
// addition: the two-sums below need the product's rounded value, and the
// kernels must evaluate every sum the same way to give the same bits.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

__device__ __forceinline__ float comp_load(const __nv_bfloat16 *c, size_t i) { return __bfloat162float(c[i]); }
__device__ __forceinline__ void comp_store(__nv_bfloat16 *c, size_t i, float x) { c[i] = __float2bfloat16_rn(x); }

// x *= g with the product's rounding error added to lo (lo scales too).
__device__ __forceinline__ void comp_scale(float &x, float &lo, float g)
{
    const float p = mul_rn(x, g);
    lo = fmaf(lo, g, fmaf(x, g, -p));
    x = p;
}

// Point-dipole loads fused into the step kernels: entry k adds
// coef[k] * g[dip[k]] to slot[k]; g for this (step n, substep q) is read at
// g + (n*nsub + q)*nd with n = ctl[par].  The entries are sorted by slot (entries
// of one slot in dipole order), so a flagged slot finds its entries by
// binary search: a linear scan of a batch's list (six entries per shot) kept
// the few warps that hold dipole slots busy long after the rest of the grid.
struct SrcArgs {
    int n;
    const int *slot;
    const double *coef;
    const int *dip;
    const double *g;
    const int *ctl;
    int nd, nsub, q;
    int par;   // the step counter of this step is ctl[par] (double-buffered by step parity)
};

__device__ __forceinline__ double source_load(const SrcArgs &s, size_t e)
{
    double f = 0.0;
    if (s.n == 0) return f;
    int lo = 0, hi = s.n;   // first entry with slot >= e
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((size_t)s.slot[mid] < e) lo = mid + 1; else hi = mid;
    }
    const double *g = s.g + ((size_t)s.ctl[s.par] * s.nsub + s.q) * s.nd;
    for (int k = lo; k < s.n && (size_t)s.slot[k] == e; ++k) f += s.coef[k] * g[s.dip[k]];
    return f;
}

// Receivers sampled inside the step launches.  The first launch of step n
// reads the step counter ctl[par] (n) and, from one block beyond the node
// blocks, records E(x) = sum_l w_l(x) U_l of every receiver when n is a
// sampling step; U is that launch's input, which no thread of the launch
// writes.  With the symplectic drifts merged the stored U holds W = U +
// h Minv P, so the sample subtracts h Minv P of the receiver slots, which
// the last launch of step n-1 left in rz (double-buffered by parity like the
// counter, so a one-launch step reads one copy and writes the other).  The
// first launch also sets ctl[1 - par] = n + 1 for the next step; no launch
// reads the copy it writes.
template <class T> struct RecArgs {
    int nrec;                  // receivers to sample at the start of this step (0: no sampling blocks)
    int nsb;                   // sampling blocks, the first of the launch
    const int *edges;          // six slot ids per receiver
    const int *rk;             // their entries in the receiver-slot list
    const double *w;           // 18 weights per receiver
    const T *rz_in;            // Minv P at the receiver slots, start of this step
    T unmerge;                 // the merged half drift (symplectic), else 0
    double *tr;
    int nsamp, tf;
    int nk;                    // receiver slots (sorted ids in kslot)
    const int *kslot;
    const int *kidx;           // per slot, its entry in kslot (read for receiver slots only)
    T *rz_out;                 // written by the step's last launch for the next step's sampling
    int *ctl;
    int par, adv;              // counter parity of this step; advance it in this launch
};

// The sampling blocks (the first nsb blocks of the launch): eight lanes per
// receiver, lane l < 6 forms its slot's terms (explicitly rounded FP64
// products), lane 0 sums them in slot order.
template <class T>
__device__ __noinline__ void sample_receivers(const RecArgs<T> rec, const T *U, size_t nnode, int tid, int nthr)
{
    const int step = rec.ctl[rec.par];
    if (step % rec.tf != 0 || step / rec.tf >= rec.nsamp) return;
    const int l = tid & 7, per = nthr >> 3;
    for (int r0 = blockIdx.x * per; r0 < rec.nrec; r0 += rec.nsb * per) {
        const int r = r0 + (tid >> 3);
        double c[3] = {0.0, 0.0, 0.0};
        if (r < rec.nrec && l < 6) {
            const size_t e = (size_t)rec.edges[6 * r + l];
            T u = U[fslot(e, nnode)];
            if (rec.unmerge != T(0)) u = fma(-rec.unmerge, rec.rz_in[rec.rk[6 * r + l]], u);
            for (int q = 0; q < 3; ++q) c[q] = __dmul_rn((double)u, rec.w[18 * r + 3 * l + q]);
        }
        double acc[3] = {0.0, 0.0, 0.0};
        for (int jl = 0; jl < 6; ++jl)
            for (int q = 0; q < 3; ++q) acc[q] = __dadd_rn(acc[q], __shfl_sync(0xffffffffu, c[q], jl, 8));
        if (r < rec.nrec && l == 0) {
            double *o = rec.tr + ((size_t)r * rec.nsamp + step / rec.tf) * 4;
            o[1] = acc[0]; o[2] = acc[1]; o[3] = acc[2];
        }
    }
}

// ------------------------------------------------------ node-centric step
// Each thread owns one node and its seven edge slots.  The tetrahedra that
// hold the node as vertex 0, 1 or 2 (the tails of its slots) sit at fixed
// cell offsets o in {-1, 0}^3 and types p: 18 around an interior node.
// Listed in ascending tetrahedron order, each feeds one to three of the
// node's slots, so every B is loaded once per node and each slot's sum runs
// over its incidences in ascending tetrahedron order (the order of the
// incidence lists).  The table is built at compile time from the Kuhn split.
struct NodeTab {
    int o[18][3], p[18];
    int ne[18], d[18][3], l[18][3];   // slots (directions) fed by entry q and their local edges
    int curl[6][6][3];                 // 2 grad(l_m) x grad(l_n) of local edge l of type p
};

constexpr NodeTab make_node_tab()
{
    NodeTab t{};
    const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    const int loc[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    const int dirs[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
    int vert[6][4][3] = {}, grad[6][4][3] = {};
    for (int p = 0; p < 6; ++p) {
        const int a = perm[p][0], b = perm[p][1], c = perm[p][2];
        vert[p][1][a] = 1;
        vert[p][2][a] = 1; vert[p][2][b] = 1;
        vert[p][3][0] = vert[p][3][1] = vert[p][3][2] = 1;
        grad[p][0][a] = -1;
        grad[p][1][a] = 1; grad[p][1][b] = -1;
        grad[p][2][b] = 1; grad[p][2][c] = -1;
        grad[p][3][c] = 1;
        for (int l = 0; l < 6; ++l) {
            const int *gm = grad[p][loc[l][0]], *gn = grad[p][loc[l][1]];
            t.curl[p][l][0] = 2 * (gm[1] * gn[2] - gm[2] * gn[1]);
            t.curl[p][l][1] = 2 * (gm[2] * gn[0] - gm[0] * gn[2]);
            t.curl[p][l][2] = 2 * (gm[0] * gn[1] - gm[1] * gn[0]);
        }
    }
    int eo[18][3] = {}, ep[18] = {}, em[18] = {};
    int n = 0;
    for (int p = 0; p < 6; ++p)
        for (int m = 0; m < 3; ++m) {
            for (int x = 0; x < 3; ++x) eo[n][x] = -vert[p][m][x];
            ep[n] = p;
            em[n] = m;
            ++n;
        }
    int idx[18] = {};
    for (int q = 0; q < 18; ++q) idx[q] = q;
    auto before = [&](int u, int w) {   // ascending tetrahedron index: cell (z, y, x), then type
        if (eo[u][2] != eo[w][2]) return eo[u][2] < eo[w][2];
        if (eo[u][1] != eo[w][1]) return eo[u][1] < eo[w][1];
        if (eo[u][0] != eo[w][0]) return eo[u][0] < eo[w][0];
        return ep[u] < ep[w];
    };
    for (int q = 1; q < 18; ++q)
        for (int r = q; r > 0 && before(idx[r], idx[r - 1]); --r) {
            const int tmp = idx[r];
            idx[r] = idx[r - 1];
            idx[r - 1] = tmp;
        }
    for (int q = 0; q < 18; ++q) {
        const int s = idx[q], p = ep[s], m = em[s];
        for (int x = 0; x < 3; ++x) t.o[q][x] = eo[s][x];
        t.p[q] = p;
        int k = 0;
        for (int l = 0; l < 6; ++l) {
            if (loc[l][0] != m) continue;
            const int *vm = vert[p][m], *vn = vert[p][loc[l][1]];
            int dd = 0;
            for (int c = 0; c < 7; ++c)
                if (dirs[c][0] == vn[0] - vm[0] && dirs[c][1] == vn[1] - vm[1] && dirs[c][2] == vn[2] - vm[2]) dd = c;
            t.d[q][k] = dd;
            t.l[q][k] = l;
            ++k;
        }
        t.ne[q] = k;
    }
    return t;
}

// ------------------------------------------------------ fused step
// The fused step recomputes the curls of a node's 18 tetrahedra from U
// instead of reading them from a per-tetrahedron array.  Their 6 x 18 edges
// are 43 distinct slots whose tails are 13 nodes at offsets in {-1,0,1}^3;
// each thread loads those 43 values once (neighbouring threads share them
// through L1/L2), so per node only U, P, the mass block, the flags and an
// 8-byte record leave DRAM.  Mask bits of a node: 1 i > 0, 2 i < nx, 4 j > 0,
// 8 j < ny, 16 k > 0, 32 k < nz; a tail node exists when the bits of its
// offset are set, a tetrahedron when the bits of its cell are.
struct StepTab {
    NodeTab n;
    int ntail, tail[13][3], treq[13];
    int nedge, etail[43], edir[43];
    int eidx[18][6];   // distinct-edge index of local edge l of entry q
    int qreq[18];      // mask bits the cell of entry q needs
    int own[7];        // distinct-edge index of the node's own slot d
    int first[7];      // entry q * 3 + component of slot d's first gather term
};

constexpr int offset_bits(int x, int y, int z)
{
    return (x < 0 ? 1 : 0) | (x > 0 ? 2 : 0) | (y < 0 ? 4 : 0) | (y > 0 ? 8 : 0) | (z < 0 ? 16 : 0) | (z > 0 ? 32 : 0);
}

constexpr StepTab make_step_tab()
{
    StepTab s{};
    s.n = make_node_tab();
    const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    const int loc[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    const int dirs[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
    int vert[6][4][3] = {};
    for (int p = 0; p < 6; ++p) {
        const int a = perm[p][0], b = perm[p][1];
        vert[p][1][a] = 1;
        vert[p][2][a] = 1; vert[p][2][b] = 1;
        vert[p][3][0] = vert[p][3][1] = vert[p][3][2] = 1;
    }
    // edge (tail offset, direction) of every local edge, and the tails in
    // ascending node order (z, y, x)
    int et[18][6][3] = {}, ed[18][6] = {};
    for (int q = 0; q < 18; ++q) {
        const int p = s.n.p[q];
        for (int l = 0; l < 6; ++l) {
            const int *vm = vert[p][loc[l][0]], *vn = vert[p][loc[l][1]];
            for (int x = 0; x < 3; ++x) et[q][l][x] = s.n.o[q][x] + vm[x];
            for (int c = 0; c < 7; ++c)
                if (dirs[c][0] == vn[0] - vm[0] && dirs[c][1] == vn[1] - vm[1] && dirs[c][2] == vn[2] - vm[2]) ed[q][l] = c;
        }
    }
    for (int z = -1; z <= 1; ++z)
        for (int y = -1; y <= 1; ++y)
            for (int x = -1; x <= 1; ++x) {
                bool used = false;
                for (int q = 0; q < 18; ++q)
                    for (int l = 0; l < 6; ++l)
                        if (et[q][l][0] == x && et[q][l][1] == y && et[q][l][2] == z) used = true;
                if (!used) continue;
                s.tail[s.ntail][0] = x; s.tail[s.ntail][1] = y; s.tail[s.ntail][2] = z;
                s.treq[s.ntail] = offset_bits(x, y, z);
                ++s.ntail;
            }
    for (int t = 0; t < s.ntail; ++t)
        for (int c = 0; c < 7; ++c) {
            bool used = false;
            for (int q = 0; q < 18; ++q)
                for (int l = 0; l < 6; ++l)
                    if (ed[q][l] == c && et[q][l][0] == s.tail[t][0] && et[q][l][1] == s.tail[t][1] && et[q][l][2] == s.tail[t][2])
                        used = true;
            if (!used) continue;
            s.etail[s.nedge] = t;
            s.edir[s.nedge] = c;
            if (s.tail[t][0] == 0 && s.tail[t][1] == 0 && s.tail[t][2] == 0) s.own[c] = s.nedge;
            ++s.nedge;
        }
    for (int d = 0; d < 7; ++d) s.first[d] = -1;
    for (int q = 0; q < 18; ++q)
        for (int k = 0; k < s.n.ne[q]; ++k)
            for (int c = 0; c < 3; ++c)
                if (s.n.curl[s.n.p[q]][s.n.l[q][k]][c] != 0 && s.first[s.n.d[q][k]] < 0) s.first[s.n.d[q][k]] = q * 3 + c;
    for (int q = 0; q < 18; ++q) {
        s.qreq[q] = (s.n.o[q][0] < 0 ? 1 : 2) | (s.n.o[q][1] < 0 ? 4 : 8) | (s.n.o[q][2] < 0 ? 16 : 32);
        for (int l = 0; l < 6; ++l)
            for (int k = 0; k < s.nedge; ++k) {
                const int t = s.etail[k];
                if (s.edir[k] == ed[q][l] && s.tail[t][0] == et[q][l][0] && s.tail[t][1] == et[q][l][1] &&
                    s.tail[t][2] == et[q][l][2])
                    s.eidx[q][l] = k;
            }
    }
    return s;
}

// Table sizes the kernel relies on (every slot of the node is an edge of
// one of its tetrahedra, so own[] is complete).
static_assert(make_step_tab().ntail == 13 && make_step_tab().nedge == 43, "Kuhn split: 13 tails, 43 edges per node");

// Contribution of entry Q of the node table (a template parameter, so every
// table index below is a compile-time constant and ue, f stay in
// registers): the curl of the tetrahedron from the edge values ue and its
// B = curl / 6 gathered into the node's slots it feeds, B . curl(w_l).
// Every curl factor of the Kuhn split is +-2, so the curl is 2 S with S a
// signed sum of edge values, B = 2 B' with B' = S / 6 rounded, and each
// gather term B . curl(w_l) component is +-4 B'; the kernel sums +-B' and
// scales the sum by 4 at the end (scaling by a power of two commutes with
// rounding, so these are the bits of the straightforward evaluation).  A
// tetrahedron outside the mesh contributes B' = 0, so every slot's first
// term is known at compile time and starts its sum without an addition.
// COMP: f is kept as hi + lo (fl): each term is added to hi by a two-sum
// whose exact error goes to lo, so the gathered force carries no rounding
// of its own.
template <class T, int Q, int COMP>
__device__ __forceinline__ void step_tet(const T (&ue)[43], T (&f)[7], T (&fl)[7], int have)
{
    constexpr StepTab tab = make_step_tab();
    constexpr int p = tab.n.p[Q];
    const bool inside = (tab.qreq[Q] & ~have) == 0;   // cell inside the mesh
    T b[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        T sum = 0;
        bool started = false;
#pragma unroll
        for (int l = 0; l < 6; ++l) {
            if (tab.n.curl[p][l][c] == 0) continue;
            const T u = ue[tab.eidx[Q][l]];
            if (!started) sum = tab.n.curl[p][l][c] > 0 ? u : -u;
            else sum = tab.n.curl[p][l][c] > 0 ? sum + u : sum - u;
            started = true;
        }
        b[c] = inside ? mul_rn(T(1.0 / 6.0), sum) : T(0);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (k < tab.n.ne[Q]) {
            const int d = tab.n.d[Q][k], l = tab.n.l[Q][k];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (tab.n.curl[p][l][c] == 0) continue;
                const T t = tab.n.curl[p][l][c] > 0 ? b[c] : -b[c];
                if (tab.first[d] == Q * 3 + c) {
                    f[d] = t;
                } else if constexpr (COMP) {
                    T e;
                    f[d] = two_sum(f[d], t, e);
                    fl[d] += e;
                } else {
                    f[d] += t;
                }
            }
        }
}

// All 18 entries in table order (ascending tetrahedron index).
template <class T, int COMP, int... Q>
__device__ __forceinline__ void step_tets(const T (&ue)[43], T (&f)[7], T (&fl)[7], int have, std::integer_sequence<int, Q...>)
{
    (step_tet<T, Q, COMP>(ue, f, fl, have), ...);
}

// Node record of the fused step: x = y-stride | mask << 26, y = z-stride (in
// nodes, within the node's shot).
__host__ __device__ constexpr int step_record_x(int sy, int mask) { return sy | (mask << 26); }

// One fused substep per node: F = K Uin gathered from the curls of its 18
// tetrahedra recomputed from Uin (curl terms over local edges 0..5, B =
// curl / 6, entries in ascending tetrahedron order, zero curl entries left
// out), then MODE 0 (symplectic) P -= a (F - f) on non-PEC slots and Uout =
// Uin + c Minv P (zout = Minv P; with minv == nullptr only P is written), or
// MODE 1 (leapfrog) Uout = 2 Uin - Uold - c Minv (F - f), PEC slots zero.
// Uout must not alias Uin: other threads read Uin around their node.
// Losses (damp per node): DAMP 1 with MODE 0 is the middle kick of a lossy
// step, P = g (g P - a (F - f)) with g = exp(-rho dt/2) (ppre, pmid, when
// given, keep P before the first factor and after the kick); DAMP 2 with
// MODE 0 is its adjoint, Uout = g Uin + c Minv P; DAMP 1 with MODE 1 is the
// lossy leapfrog, Uout = (2 Uin - (1 - r) Uold - c Minv (F - f)) / (1 + r)
// with r = rho dt / 2.  REC (the last launch of a symplectic step) also
// keeps Minv P of the receiver slots in rec.rz_out.  COMP (FP32, MODE 0)
// adds the kick and drift increments by compensated sums with the bfloat16
// plane cmp.p (see "compensated updates"); the loss factors
// scale lo with hi.
// Threads per block of the fused step: chosen per handle by timing these
// candidates on the handle's own mesh (TetFemSim::force_launch_shape); small
// meshes (a 32^3 mesh has 36k nodes) spread better over the 152 SMs in
// small blocks.  The block size changes no arithmetic.
constexpr int kStepBlocks[4] = {32, 64, 128, 256};
constexpr int kStepBlockMax = 256;

template <class T, int MODE, int DAMP, int REC = 0, int COMP = 0>
__global__ void __launch_bounds__(kStepBlockMax) tet_step_kernel(size_t nnode, const int2 *__restrict__ nrec,
                                                       const unsigned char *__restrict__ pec, const T *__restrict__ minv,
                                                       T *__restrict__ P, const T *__restrict__ Uin, T *__restrict__ Uout,
                                                       const T *__restrict__ Uold, T a, T c, SrcArgs src, T *__restrict__ zout,
                                                       const T *__restrict__ damp, T *__restrict__ ppre, T *__restrict__ pmid,
                                                       RecArgs<T> rec, Comp cmp)
{
    static_assert(!COMP || (MODE == 0 && std::is_same<T, float>::value), "compensated updates: FP32 symplectic steps");
    constexpr StepTab tab = make_step_tab();
    // the first rec.nsb blocks sample the receivers when this launch does
    // (they run in the first wave, beside the node blocks); the node blocks
    // follow them
    const int nb = (int)blockIdx.x - rec.nsb;
    if (nb < 0) {
        sample_receivers<T>(rec, Uin, nnode, (int)threadIdx.x, (int)blockDim.x);
        return;
    }
    const size_t v = (size_t)nb * blockDim.x + threadIdx.x;
    if (v >= nnode) return;
    if (rec.adv && v == 0) rec.ctl[1 - rec.par] = rec.ctl[rec.par] + 1;
    const int2 r = __ldg(nrec + v);
    const int have = (int)((unsigned)r.x >> 26), sy = r.x & 0x3ffffff, sz = r.y;
    const T *u0 = Uin + v;
    // a missing tail node only feeds missing tetrahedra: read the node's own
    // slots instead (in bounds) and let the cell test drop them
    int off[13];
#pragma unroll
    for (int t = 0; t < 13; ++t)
        off[t] = (tab.treq[t] & ~have) == 0 ? tab.tail[t][0] + tab.tail[t][1] * sy + tab.tail[t][2] * sz : 0;
    T ue[43];
#pragma unroll
    for (int k = 0; k < 43; ++k) ue[k] = u0[(size_t)tab.edir[k] * nnode + off[tab.etail[k]]];
    T f[7] = {0, 0, 0, 0, 0, 0, 0}, fl[7] = {0, 0, 0, 0, 0, 0, 0};
    step_tets<T, COMP>(ue, f, fl, have, std::make_integer_sequence<int, 18>{});
#pragma unroll
    for (int d = 0; d < 7; ++d) { f[d] *= T(4); fl[d] *= T(4); }
    const size_t e0 = 7 * v;   // the node's slots in the flag table and the source list
    unsigned char m[7];
    T x[7], u[7];
    const T g = DAMP ? damp[v] : T(1);
    int recmask = 0;   // the node's receiver slots (REC)
#pragma unroll
    for (int d = 0; d < 7; ++d) {
        m[d] = pec[e0 + d];
        if (REC && (m[d] & kRecBit)) recmask |= 1 << d;
        u[d] = ue[tab.own[d]];
        if (MODE == 0) x[d] = P[(size_t)d * nnode + v];
    }
#pragma unroll
    for (int d = 0; d < 7; ++d) {
        const size_t f0 = (size_t)d * nnode + v;
        if constexpr (COMP) {
            T lp = comp_load(cmp.p, f0);
            if (DAMP == 1) {
                if (ppre) ppre[f0] = x[d];
                comp_scale(x[d], lp, g);
            }
            if (!(m[d] & kPecBit)) {
                // P + lo - a (f + fl) + a s as hi + lo: the product -a f
                // split exactly into p1 and its error, the small terms summed
                // into t, then two exact sums
                const T p1 = mul_rn(-a, f[d]);
                T t = fma(-a, f[d], -p1) + lp;
                t = fma(-a, fl[d], t);
                if (m[d] & kSrcBit) t = fma(a, (T)source_load(src, e0 + d), t);
                T e;
                const T s1 = two_sum(x[d], p1, e);
                x[d] = two_sum(s1, t + e, lp);
            }
            if (DAMP == 1) {
                if (pmid) pmid[f0] = x[d];
                comp_scale(x[d], lp, g);
            }
            P[f0] = x[d];
            comp_store(cmp.p, f0, lp);
        } else if (MODE == 0) {
            if (DAMP == 1) {
                if (ppre) ppre[f0] = x[d];
                x[d] *= g;
            }
            if (!(m[d] & kPecBit)) {
                x[d] = fma(-a, f[d], x[d]);
                if (m[d] & kSrcBit) x[d] = fma(a, (T)source_load(src, e0 + d), x[d]);
            }
            if (DAMP == 1) {
                if (pmid) pmid[f0] = x[d];
                x[d] *= g;
            }
            P[f0] = x[d];
        } else {
            x[d] = T(0);
            if (!(m[d] & kPecBit)) {
                x[d] = f[d];
                if (m[d] & kSrcBit) x[d] -= (T)source_load(src, e0 + d);
            }
        }
    }
    if (minv == nullptr) return;   // force-only use (uniform across the grid)
    T mv[28];
    load_block<T>(minv, nnode, v, mv);
#pragma unroll
    for (int d = 0; d < 7; ++d) {
        const size_t f0 = (size_t)d * nnode + v;
        const T y = block_row<T>(mv, x, d);
        if (MODE == 0) {
            Uout[f0] = fma(c, y, DAMP == 2 ? g * u[d] : u[d]);
            if (zout) zout[f0] = y;
            if (REC && ((recmask >> d) & 1)) rec.rz_out[rec.kidx[e0 + d]] = y;
        } else if (DAMP) {
            Uout[f0] = (m[d] & kPecBit) ? T(0) : (fma(-c, y, T(2) * u[d]) - (T(1) - g) * Uold[f0]) / (T(1) + g);
        } else {
            Uout[f0] = (m[d] & kPecBit) ? T(0) : fma(-c, y, T(2) * u[d] - Uold[f0]);
        }
    }
}

// ------------------------------------------------------ slot-split step
// One thread per node gives a mesh held in L2 (a 32^3 mesh has 36k nodes)
// about seven warps per SM, too few to hide the latency of the neighbour
// loads.  The slot-split step runs seven warps per 32 nodes: warp d takes
// slot d of its 32 nodes.  It reads the edge values of the tetrahedra that
// hold the slot's edge, forms only the curl components the slot's gather
// needs, gathers the slot's force and kicks P_d; after a block barrier it
// forms (Minv P)_d from the node's seven kicked P values in shared memory
// and drifts U_d.  Every sum runs in the order of the node kernel (entries
// ascending, components ascending, the mass row in column order), so both
// kernels give the same bits.  MODE 0 without losses only.
constexpr int kSlotNodes = 32;               // nodes per block (one per lane)
constexpr int kSlotThreads = 7 * kSlotNodes; // the block: one warp per slot direction

struct SlotTab {
    int nt[7];          // node-table entries whose tetrahedron holds slot d's edge
    int q[7][6];        // those entries, ascending
    int l[7][6];        // the local edge of slot d in each
    int nu[7];          // distinct edge values slot d reads
    int ue[7][36];      // their indices in the 43-edge list of StepTab
    int ui[7][6][6];    // local edge l' of feed k -> index into the slot's values (-1: not read)
};

constexpr SlotTab make_slot_tab()
{
    SlotTab s{};
    const StepTab t = make_step_tab();
    for (int d = 0; d < 7; ++d) {
        for (int q = 0; q < 18; ++q)
            for (int k = 0; k < t.n.ne[q]; ++k)
                if (t.n.d[q][k] == d) {
                    s.q[d][s.nt[d]] = q;
                    s.l[d][s.nt[d]] = t.n.l[q][k];
                    ++s.nt[d];
                }
        for (int k = 0; k < s.nt[d]; ++k) {
            const int q = s.q[d][k], p = t.n.p[q], l = s.l[d][k];
            for (int l2 = 0; l2 < 6; ++l2) {
                s.ui[d][k][l2] = -1;
                bool need = false;   // l2 enters a curl component that the gather of slot d uses
                for (int c = 0; c < 3; ++c)
                    if (t.n.curl[p][l][c] != 0 && t.n.curl[p][l2][c] != 0) need = true;
                if (!need) continue;
                const int e = t.eidx[q][l2];
                int at = -1;
                for (int u = 0; u < s.nu[d]; ++u)
                    if (s.ue[d][u] == e) at = u;
                if (at < 0) { at = s.nu[d]; s.ue[d][s.nu[d]++] = e; }
                s.ui[d][k][l2] = at;
            }
        }
    }
    return s;
}

// Feed K of slot D: the curl components of that tetrahedron that the gather
// of slot D needs, B' = S / 6 (zero outside the mesh), and their terms
// +-B' added to f in component order (the first term of the slot starts the
// sum).  Template parameters make every table index a constant.
template <class T, int D, int K, int COMP, int NU>
__device__ __forceinline__ void slot_feed(const T (&ue)[NU], int have, T &f, T &fl)
{
    constexpr StepTab tab = make_step_tab();
    constexpr SlotTab st = make_slot_tab();
    constexpr int q = st.q[D][K], p = tab.n.p[q], l = st.l[D][K];
    const bool inside = (tab.qreq[q] & ~have) == 0;
    bool first = K == 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (tab.n.curl[p][l][c] == 0) continue;
        T sum = 0;
        bool started = false;
#pragma unroll
        for (int l2 = 0; l2 < 6; ++l2) {
            if (tab.n.curl[p][l2][c] == 0) continue;
            const T u = ue[st.ui[D][K][l2]];
            if (!started) sum = tab.n.curl[p][l2][c] > 0 ? u : -u;
            else sum = tab.n.curl[p][l2][c] > 0 ? sum + u : sum - u;
            started = true;
        }
        const T b = inside ? mul_rn(T(1.0 / 6.0), sum) : T(0);
        const T t = tab.n.curl[p][l][c] > 0 ? b : -b;
        if (first) {
            f = t;
            first = false;
        } else if constexpr (COMP) {
            T e;
            f = two_sum(f, t, e);
            fl += e;
        } else {
            f += t;
        }
    }
}

template <class T, int D, int COMP, int NU, int... K>
__device__ __forceinline__ void slot_feeds(const T (&ue)[NU], int have, T &f, T &fl, std::integer_sequence<int, K...>)
{
    (slot_feed<T, D, K, COMP, NU>(ue, have, f, fl), ...);
}

// u0 carries no __restrict__: the persistent step reads U buffers that
// other blocks of the same launch wrote before a grid barrier, so its loads
// must not take the non-coherent read-only path.
// I: the index type (size_t, or int where every slot index fits in 31 bits).
template <class T, int D, int NU, class I, int... K>
__device__ __forceinline__ void slot_loads(T (&ue)[NU], const T *u0, I nnode, const int (&off)[13],
                                           std::integer_sequence<int, K...>)
{
    constexpr StepTab tab = make_step_tab();
    constexpr SlotTab st = make_slot_tab();
    ((ue[K] = u0[(I)tab.edir[st.ue[D][K]] * nnode + off[tab.etail[st.ue[D][K]]]]), ...);
}

// Row D of the node's packed mass block (plane layout), in column order.
template <class T, int D, int... J>
__device__ __forceinline__ void slot_mass_row(const T *__restrict__ minv, size_t v, size_t nnode, T (&row)[7],
                                              std::integer_sequence<int, J...>)
{
    constexpr int idx[7] = {(D < J ? D * (13 - D) / 2 + J : J * (13 - J) / 2 + D)...};   // packed (D, j)
    ((row[J] = minv[fpk(v, idx[J], nnode)]), ...);
}

// Force of slot D of one node, f = K U restricted to the slot, as hi + lo
// with COMP (see step_tet).
template <class T, int D, int COMP, class I>
__device__ __forceinline__ void slot_curl(const T *u0, I nnode, const int (&off)[13], int have, T &f, T &fl)
{
    constexpr SlotTab st = make_slot_tab();
    constexpr int nu = st.nu[D], nt = st.nt[D];
    T ue[nu];
    slot_loads<T, D, nu>(ue, u0, nnode, off, std::make_integer_sequence<int, nu>{});
    f = 0;
    fl = 0;
    slot_feeds<T, D, COMP, nu>(ue, have, f, fl, std::make_integer_sequence<int, nt>{});
    f *= T(4);
    fl *= T(4);
}

// The force of slot D and row D of the node's mass block.
template <class T, int D, int COMP>
__device__ __forceinline__ void slot_force(const T *u0, size_t nnode, const int (&off)[13], int have, T &f, T &fl,
                                           const T *__restrict__ minv, size_t v, T (&row)[7])
{
    slot_mass_row<T, D>(minv, v, nnode, row, std::make_integer_sequence<int, 7>{});
    slot_curl<T, D, COMP>(u0, nnode, off, have, f, fl);
}

// FP32: at most 32 registers, so 8 blocks fit on an SM and the 1,125 blocks
// of the 32^3 headline mesh run in one wave (40 registers left 61 blocks
// for a second wave; 30.7 -> 29.8 ms per 2000-step solve).
template <class T, int REC, int COMP>
__global__ void __launch_bounds__(kSlotThreads, sizeof(T) == 4 ? 8 : 1) tet_slot_kernel(size_t nnode, const int2 *__restrict__ nrec,
                                                                const unsigned char *__restrict__ pec,
                                                                const T *__restrict__ minv, T *__restrict__ P,
                                                                const T *__restrict__ Uin, T *__restrict__ Uout, T a, T c,
                                                                SrcArgs src, T *__restrict__ zout, RecArgs<T> rec, Comp cmp)
{
    constexpr StepTab tab = make_step_tab();
    const int nb = (int)blockIdx.x - rec.nsb;
    if (nb < 0) {   // the leading blocks sample the receivers (no barrier below is reached)
        sample_receivers<T>(rec, Uin, nnode, (int)(threadIdx.y * kSlotNodes + threadIdx.x), kSlotThreads);
        return;
    }
    __shared__ T sx[7][kSlotNodes];
    const int lane = threadIdx.x, d = threadIdx.y;
    const size_t v = (size_t)nb * kSlotNodes + lane;
    const bool valid = v < nnode;
    if (rec.adv && v == 0 && d == 0) rec.ctl[1 - rec.par] = rec.ctl[rec.par] + 1;
    const size_t f0 = (size_t)d * nnode + v, e0 = 7 * v;
    T x = 0, u = 0, row[7] = {0, 0, 0, 0, 0, 0, 0};   // row: the mass row of slot d, loaded before the barrier
    unsigned char m = 0;
    if (valid) {
        const int2 r = __ldg(nrec + v);
        const int have = (int)((unsigned)r.x >> 26), sy = r.x & 0x3ffffff, sz = r.y;
        int off[13];
#pragma unroll
        for (int t = 0; t < 13; ++t)
            off[t] = (tab.treq[t] & ~have) == 0 ? tab.tail[t][0] + tab.tail[t][1] * sy + tab.tail[t][2] * sz : 0;
        T f = 0, fl = 0;
        const T *u0 = Uin + v;
        switch (d) {   // warp-uniform: warp d runs slot d
        case 0: slot_force<T, 0, COMP>(u0, nnode, off, have, f, fl, minv, v, row); break;
        case 1: slot_force<T, 1, COMP>(u0, nnode, off, have, f, fl, minv, v, row); break;
        case 2: slot_force<T, 2, COMP>(u0, nnode, off, have, f, fl, minv, v, row); break;
        case 3: slot_force<T, 3, COMP>(u0, nnode, off, have, f, fl, minv, v, row); break;
        case 4: slot_force<T, 4, COMP>(u0, nnode, off, have, f, fl, minv, v, row); break;
        case 5: slot_force<T, 5, COMP>(u0, nnode, off, have, f, fl, minv, v, row); break;
        default: slot_force<T, 6, COMP>(u0, nnode, off, have, f, fl, minv, v, row); break;
        }
        u = Uin[f0];
        m = pec[e0 + d];
        x = P[f0];
        // the kick of the node kernel (MODE 0, no losses)
        if constexpr (COMP) {
            T lp = comp_load(cmp.p, f0);
            if (!(m & kPecBit)) {
                const T p1 = mul_rn(-a, f);
                T t = fma(-a, f, -p1) + lp;
                t = fma(-a, fl, t);
                if (m & kSrcBit) t = fma(a, (T)source_load(src, e0 + d), t);
                T e;
                const T s1 = two_sum(x, p1, e);
                x = two_sum(s1, t + e, lp);
            }
            comp_store(cmp.p, f0, lp);
        } else {
            if (!(m & kPecBit)) {
                x = fma(-a, f, x);
                if (m & kSrcBit) x = fma(a, (T)source_load(src, e0 + d), x);
            }
        }
        P[f0] = x;
    }
    sx[d][lane] = x;
    __syncthreads();
    if (!valid) return;
    T y = 0;
#pragma unroll
    for (int j = 0; j < 7; ++j) y = fma(row[j], sx[j][lane], y);
    Uout[f0] = fma(c, y, u);
    if (zout) zout[f0] = y;
    if (REC && (m & kRecBit)) rec.rz_out[rec.kidx[e0 + d]] = y;
}

// ------------------------------------------------------ persistent step
// A grid barrier with a bounded wait, for kernels launched cooperatively
// (every block resident).  Block 0 adds 2^31 - (expected - 1) to the
// arrival counter, every other block 1: the counter's top bit flips when
// the last block arrives and its low bits return to zero, so the barrier
// resets itself.  One thread per block polls for the flip (relaxed loads;
// the fence after the last one makes the wait an acquire) at most limit_ns
// and at most kBarrierPolls times, then sets err and returns false; so
// does every block that finds err set while it waits.  A launch whose
// barrier cannot complete therefore ends within about limit_ns, and the
// host reads err.
struct GridBarrier {
    unsigned *count;               // arrivals (zero before the first launch of a run)
    int *err;                      // nonzero: a wait gave up
    unsigned expected;             // blocks that arrive at every barrier
    unsigned long long limit_ns;   // longest wait of one block
};
constexpr unsigned kBarrierPolls = 1u << 24;

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned load_relaxed(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ bool grid_barrier(const GridBarrier &b, int *ok_sh)
{
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        const unsigned add = blockIdx.x == 0 ? 0x80000000u - (b.expected - 1u) : 1u;
        __threadfence();   // the block's writes (ordered by the block barrier) before the arrival
        const unsigned old = atomicAdd(b.count, add);
        int ok = 1;
        const unsigned long long t0 = global_ns();
        for (unsigned it = 0; ((load_relaxed(b.count) ^ old) & 0x80000000u) == 0; ++it) {
            if (*(volatile int *)b.err != 0 || it >= kBarrierPolls || ((it & 31) == 31 && global_ns() - t0 > b.limit_ns)) {
                atomicExch(b.err, 1);
                ok = 0;
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
        *ok_sh = ok;
    }
    __syncthreads();
    return *ok_sh != 0;
}

// Arguments of the persistent step.
template <class T> struct PersistArgs {
    T *U[2];                  // substep k of the launch reads U[k & 1] and writes U[(k + 1) & 1]
    T *P;
    __nv_bfloat16 *cp;        // P's compensation plane (COMP)
    T a[3], c[3];             // kick and merged drift lengths of the substeps
    int nsub, nsteps, par0;   // substeps per step, steps of the launch, counter parity of its first step
    T *rz;                    // Minv P at the receiver slots: two copies of nrz, by counter parity
    int nrz, keep_rz;         // keep_rz: the last substep of a step writes the next step's copy
    GridBarrier bar;
};

// nsteps symplectic lossless steps in one cooperative launch: the
// slot-split step of tet_slot_kernel, with a grid barrier between
// substeps instead of a launch boundary.  Each block owns one 32-node unit
// for the whole launch (the grid covers the mesh in one wave), so the
// node's record, slot flags and mass row are read once per launch, and P,
// its compensation and the slot's own U value stay in shared memory
// between substeps (P in the exchange array the drift reads; the bfloat16
// rounding of the compensation plane applied where tet_slot_kernel stores
// it).  The first rec.nsb blocks sample the receivers at the start of every
// step; block 0's first thread advances the step counter as the first
// launch of a step does.  Every sum is the slot kernel's, so both give the
// same bits.
template <class T, int COMP>
__global__ void __launch_bounds__(kSlotThreads, sizeof(T) == 4 ? 8 : 1) tet_persist_kernel(size_t nnode, const int2 *__restrict__ nrec,
                                                                   const unsigned char *__restrict__ pec,
                                                                   const T *__restrict__ minv, PersistArgs<T> pa,
                                                                   SrcArgs src, RecArgs<T> rec)
{
    static_assert(!COMP || std::is_same<T, float>::value, "compensated updates: FP32");
    constexpr StepTab tab = make_step_tab();
    __shared__ T srow[7][7][kSlotNodes];   // the mass rows: [slot][column][node]
    __shared__ T sx[7][kSlotNodes];        // P (the drift reads the node's seven values)
    __shared__ T su[7][kSlotNodes];        // the slot's own U value
    __shared__ T slo[COMP ? 7 : 1][kSlotNodes];   // P's compensation (bfloat16 values)
    __shared__ int2 srec[kSlotNodes];      // the node records
    __shared__ unsigned char sm[7][kSlotNodes];   // slot flags
    __shared__ int sok;
    const int lane = threadIdx.x, d = threadIdx.y;
    const int nb = (int)blockIdx.x - rec.nsb;
    if (nb < 0) {   // a sampling block: the receivers at the start of every step
        int k = 0;
        for (int s = 0; s < pa.nsteps; ++s)
            for (int q = 0; q < pa.nsub; ++q, ++k) {
                if (k > 0 && !grid_barrier(pa.bar, &sok)) return;
                if (q == 0) {
                    RecArgs<T> r = rec;
                    r.par = (pa.par0 + s) & 1;
                    r.rz_in = pa.rz + (size_t)r.par * pa.nrz;
                    sample_receivers<T>(r, (k & 1) ? pa.U[1] : pa.U[0], nnode, d * kSlotNodes + lane, kSlotThreads);
                }
            }
        return;
    }
    const int nn = (int)nnode;   // slot indices fit in 31 bits
    const int v = nb * kSlotNodes + lane;
    const bool valid = v < nn;
    if (valid) {
        const int f0 = d * nn + v;
        if (d == 0) srec[lane] = __ldg(nrec + v);
        T row[7];
        switch (d) {
        case 0: slot_mass_row<T, 0>(minv, v, nnode, row, std::make_integer_sequence<int, 7>{}); break;
        case 1: slot_mass_row<T, 1>(minv, v, nnode, row, std::make_integer_sequence<int, 7>{}); break;
        case 2: slot_mass_row<T, 2>(minv, v, nnode, row, std::make_integer_sequence<int, 7>{}); break;
        case 3: slot_mass_row<T, 3>(minv, v, nnode, row, std::make_integer_sequence<int, 7>{}); break;
        case 4: slot_mass_row<T, 4>(minv, v, nnode, row, std::make_integer_sequence<int, 7>{}); break;
        case 5: slot_mass_row<T, 5>(minv, v, nnode, row, std::make_integer_sequence<int, 7>{}); break;
        default: slot_mass_row<T, 6>(minv, v, nnode, row, std::make_integer_sequence<int, 7>{}); break;
        }
#pragma unroll
        for (int j = 0; j < 7; ++j) srow[d][j][lane] = row[j];
        sm[d][lane] = pec[7 * v + d];
        sx[d][lane] = pa.P[f0];
        su[d][lane] = pa.U[0][f0];
        if constexpr (COMP) slo[d][lane] = comp_load(pa.cp, f0);
    } else {
        sx[d][lane] = T(0);
    }
    __syncthreads();
    int k = 0;   // substep of the launch
    for (int s = 0; s < pa.nsteps; ++s) {
        const int par = (pa.par0 + s) & 1;
        for (int q = 0; q < pa.nsub; ++q, ++k) {
            if (k > 0 && !grid_barrier(pa.bar, &sok)) return;
            // selects, not indexing: a runtime index into the parameter
            // arrays would copy them to local memory
            const T *Uin = (k & 1) ? pa.U[1] : pa.U[0];
            if (q == 0 && rec.adv && v == 0 && d == 0) rec.ctl[1 - par] = rec.ctl[par] + 1;
            if (valid) {
                const int2 r = srec[lane];
                const int have = (int)((unsigned)r.x >> 26), sy = r.x & 0x3ffffff, sz = r.y;
                int off[13];
#pragma unroll
                for (int t = 0; t < 13; ++t)
                    off[t] = (tab.treq[t] & ~have) == 0 ? tab.tail[t][0] + tab.tail[t][1] * sy + tab.tail[t][2] * sz : 0;
                T f = 0, fl = 0;
                const T *u0 = Uin + v;
                switch (d) {
                case 0: slot_curl<T, 0, COMP>(u0, nn, off, have, f, fl); break;
                case 1: slot_curl<T, 1, COMP>(u0, nn, off, have, f, fl); break;
                case 2: slot_curl<T, 2, COMP>(u0, nn, off, have, f, fl); break;
                case 3: slot_curl<T, 3, COMP>(u0, nn, off, have, f, fl); break;
                case 4: slot_curl<T, 4, COMP>(u0, nn, off, have, f, fl); break;
                case 5: slot_curl<T, 5, COMP>(u0, nn, off, have, f, fl); break;
                default: slot_curl<T, 6, COMP>(u0, nn, off, have, f, fl); break;
                }
                const unsigned char m = sm[d][lane];
                if (!(m & kPecBit)) {
                    const T a = q == 0 ? pa.a[0] : q == 1 ? pa.a[1] : pa.a[2];
                    T sv = 0;
                    if (m & kSrcBit) {
                        SrcArgs sq = src;
                        sq.q = q;
                        sq.par = par;
                        sv = (T)source_load(sq, 7 * v + d);
                    }
                    T x = sx[d][lane];
                    if constexpr (COMP) {
                        T lp = slo[d][lane];
                        const T p1 = mul_rn(-a, f);
                        T t = fma(-a, f, -p1) + lp;
                        t = fma(-a, fl, t);
                        if (m & kSrcBit) t = fma(a, sv, t);
                        T e;
                        const T s1 = two_sum(x, p1, e);
                        x = two_sum(s1, t + e, lp);
                        slo[d][lane] = __bfloat162float(__float2bfloat16_rn(lp));   // the plane holds bfloat16
                    } else {
                        x = fma(-a, f, x);
                        if (m & kSrcBit) x = fma(a, sv, x);
                    }
                    sx[d][lane] = x;
                }
            }
            __syncthreads();
            if (valid) {
                T y = 0;
#pragma unroll
                for (int j = 0; j < 7; ++j) y = fma(srow[d][j][lane], sx[j][lane], y);
                const T u = fma(q == 0 ? pa.c[0] : q == 1 ? pa.c[1] : pa.c[2], y, su[d][lane]);
                su[d][lane] = u;
                ((k & 1) ? pa.U[0] : pa.U[1])[d * nn + v] = u;
                if (pa.keep_rz && q == pa.nsub - 1 && (sm[d][lane] & kRecBit))
                    pa.rz[(size_t)(1 - par) * pa.nrz + rec.kidx[7 * v + d]] = y;
            }
        }
    }
    if (valid) {
        const int f0 = d * nn + v;
        pa.P[f0] = sx[d][lane];
        if constexpr (COMP) comp_store(pa.cp, f0, slo[d][lane]);
    }
}

// Adjoint of the second loss factor of a lossy middle kick and the loss
// sensitivities of both factors (node-local, before the adjoint kick):
// with Pbar the sensitivity to P after the kick's second factor,
// zr_v += Pbar . Pmid + (g Pbar) . Ppre in FP64 (the sensitivity after the
// first factor is g Pbar, the adjoint kick leaves Pbar alone), Pbar = g Pbar.
template <class T>
__global__ void __launch_bounds__(128) tet_loss_adjoint_kernel(size_t nnode, const T *__restrict__ damp, T *__restrict__ Pb,
                                                               const T *__restrict__ pmid, const T *__restrict__ ppre,
                                                               double *__restrict__ zr)
{
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nnode) return;
    const T g = damp[v];
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < 7; ++d) {
        const size_t e = (size_t)d * nnode + v;
        const T pb = Pb[e], pg = g * pb;
        s = fma((double)pb, (double)pmid[e], s);
        s = fma((double)pg, (double)ppre[e], s);
        Pb[e] = pg;
    }
    zr[v] += s;
}

// Minv P at the receiver slots (rz for the sampling at the start of a run
// or of a recomputed segment), the arithmetic of the step kernel's drift.
template <class T>
__global__ void tet_rz_init_kernel(int nk, const int *__restrict__ kslot, size_t nnode, const T *__restrict__ minv,
                                   const T *__restrict__ P, T *__restrict__ rz)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    const size_t e = (size_t)kslot[k], v = e / 7;
    T x[7], mv[28];
#pragma unroll
    for (int j = 0; j < 7; ++j) x[j] = P[(size_t)j * nnode + v];
    load_block<T>(minv, nnode, v, mv);
    rz[k] = block_row<T>(mv, x, (int)(e % 7));
}

// U += c * Minv P (drift alone), one thread per node.
template <class T>
__global__ void __launch_bounds__(128) tet_drift_kernel(size_t nnode, const T *__restrict__ minv, const T *__restrict__ P,
                                                        T *__restrict__ U, T c)
{
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nnode) return;
    T x[7], mv[28];
#pragma unroll
    for (int d = 0; d < 7; ++d) x[d] = P[(size_t)d * nnode + v];
    load_block<T>(minv, nnode, v, mv);
#pragma unroll
    for (int d = 0; d < 7; ++d) {
        const size_t f0 = (size_t)d * nnode + v;
        U[f0] = fma(c, block_row<T>(mv, x, d), U[f0]);
    }
}

// ---------------------------------------------------------------- adjoint
// The discrete adjoint of the merged symplectic loop runs the same step
// launch per substep backward in time.  Only the mass blocks depend on
// eps, so each drift U += c Minv P adds
// -c (Minv Ubar)^T dM (Minv P) to dJ/deps.  The adjoint substep is the
// forward one with the roles swapped (curl of Pbar, kick on Ubar, drift on
// Pbar; Pbar alternates between two buffers like U), storing y = Minv Ubar
// of every drift of a segment next to the forward z = Minv P;
// tet_grad_accumulate_kernel then sums the outer products per node
// (Q_v += c sym(y z^T), FP64, packed symmetric like the mass blocks) in one
// streaming pass per segment, and tet_grad_node_kernel contracts Q with
// dM_v/deps once at the end.

// Q_v += sum_k c_k sym(y_k z_k^T) over the nk drifts of one segment, one
// thread per node (28 packed entries).  Drift k = nsub * i + q of the
// segment starting at step n0 has the coefficient cq[q - 1] (q > 0),
// cq[nsub - 1] (q = 0, step > 0) or hfirst (the initial half drift).  The
// products of kAccSteps time steps are summed in T, those partial sums in
// FP64.  At GB300's FP64 rate folding every step made the pass FP64-bound
// (0.79 s of a 3.2 s backward for 16 shots on 48^3 meshes); every four
// steps it takes 0.33 s, and the FP32-vs-FP64 gradient error stays at
// 3.9e-7.
constexpr int kAccSteps = 4;

template <class T>
__global__ void __launch_bounds__(128) tet_grad_accumulate_kernel(size_t nnode, size_t nslot, int nk, int nsub, int n0,
                                                                  T c0, T c1, T c2, T hfirst, const T *__restrict__ ybuf,
                                                                  const T *__restrict__ zbuf, double *__restrict__ Q)
{
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nnode) return;
    double acc[28];
    T part[28];
#pragma unroll
    for (int p = 0; p < 28; ++p) { acc[p] = 0.0; part[p] = T(0); }
    const T clast = nsub == 3 ? c2 : (nsub == 2 ? c1 : c0);   // cq[nsub - 1]
    for (int k = 0; k < nk; ++k) {
        const int q = k % nsub;
        const T c = q > 0 ? (q == 1 ? c0 : c1) : (n0 + k / nsub > 0 ? clast : hfirst);
        T y[7], z[7];
#pragma unroll
        for (int d = 0; d < 7; ++d) {
            y[d] = ybuf[(size_t)k * nslot + (size_t)d * nnode + v];
            z[d] = zbuf[(size_t)k * nslot + (size_t)d * nnode + v];
        }
#pragma unroll
        for (int d = 0; d < 7; ++d)
#pragma unroll
            for (int j = d; j < 7; ++j) {
                const int p = d * (13 - d) / 2 + j;
                part[p] = fma(c, fma(y[d], z[j], y[j] * z[d]), part[p]);
            }
        if ((k + 1) % (nsub * kAccSteps) == 0 || k == nk - 1) {
#pragma unroll
            for (int p = 0; p < 28; ++p) { acc[p] += (double)part[p]; part[p] = T(0); }
        }
    }
    double *qv = Q + 28 * v;
#pragma unroll
    for (int p = 0; p < 28; ++p) qv[p] += 0.5 * acc[p];
}

// Receiver adjoint of one sample, in two launches.  The receivers' edge
// slots are listed once each: tet_receiver_gather_kernel gathers w * r over
// each slot's receiver terms (a, also added to Wbar); then every node
// holding such a slot gets the half drift that the merged loop folded into
// the sampling, Pbar += cc Minv a, Q += cc sym((Minv a) z^T), one thread per
// node in tet_receiver_drift_kernel.  (On one block the node part was
// bound by a single SM's FP64 rate: about 37 us per sample for 512
// receivers.)
template <class T>
__global__ void __launch_bounds__(256) tet_receiver_gather_kernel(int nsl, const int *__restrict__ sl_slot,
                                                                  const int *__restrict__ sl_ptr, const int *__restrict__ term_rc,
                                                                  const double *__restrict__ term_w, const double *__restrict__ r,
                                                                  double *__restrict__ a_scr, T *__restrict__ Wb, size_t nnode)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nsl) return;
    double acc = 0.0;
    for (int s = sl_ptr[k]; s < sl_ptr[k + 1]; ++s) acc += term_w[s] * r[term_rc[s]];
    a_scr[k] = acc;
    Wb[fslot((size_t)sl_slot[k], nnode)] += (T)acc;
}

template <class T>
__global__ void __launch_bounds__(128) tet_receiver_drift_kernel(int nnd, const int *__restrict__ nd_node,
                                                                 const int *__restrict__ nd_map, const double *__restrict__ a_scr,
                                                                 T *__restrict__ Pb, const T *__restrict__ minv,
                                                                 const T *__restrict__ z, double *__restrict__ Q, double cc,
                                                                 size_t nnode)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nnd) return;
    const size_t v = (size_t)nd_node[i];
    T x[7], y[7], zz[7];
    for (int d = 0; d < 7; ++d) {
        int k = nd_map[7 * i + d];
        x[d] = k >= 0 ? (T)a_scr[k] : T(0);
        zz[d] = z[(size_t)d * nnode + v];
    }
    for (int d = 0; d < 7; ++d) {
        T s = 0;
        for (int j = 0; j < 7; ++j) s = fma(minv[fpk(v, pk7(d, j), nnode)], x[j], s);
        y[d] = s;
        Pb[(size_t)d * nnode + v] = fma((T)cc, s, Pb[(size_t)d * nnode + v]);
    }
    for (int d = 0; d < 7; ++d)
        for (int j = d; j < 7; ++j)
            Q[28 * v + pk7(d, j)] += 0.5 * cc * ((double)y[d] * (double)zz[j] + (double)y[j] * (double)zz[d]);
}

// dJ/deps contributions of node v, FP64.  With M_v = W S^+ W^T +
// alpha (I - D G^+ D^T) and Q_v over the live slots,
//   -<dM_v/deps_t, Q_v> = -sum over the incidences (slot r, tet t, edge l) of
//       2 wint_l . Z_r + D_r^T Y wint_l + wsq_l pq,
//   Z = Q W S^+,  pq = <I - D G^+ D^T, Q> / k,  Y = V (F o V^T (W^T Q W) V) V^T,
// where V, lambda diagonalise S, S^+ keeps lambda > 1e-10 max|lambda|, and
// F holds the divided differences of f(lambda) = 1/lambda (kept) or 0
// (dropped), the derivative of that spectral function.  One value per
// incidence entry, written to contrib at the entry's position.
__global__ void tet_grad_node_kernel(size_t nnode, const unsigned char *__restrict__ pec, const int *__restrict__ inc_ptr,
                                     const int *__restrict__ inc, const double *__restrict__ eps,
                                     const double *__restrict__ Q, double *__restrict__ contrib)
{
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nnode) return;
    int slot[7], k = 0;
    for (int d = 0; d < 7; ++d)
        if (!(pec[7 * v + d] & kPecBit)) slot[k++] = d;
    if (k == 0) return;
    double W[7][3], D[7][3];
    for (int r = 0; r < k; ++r) {
        size_t e = 7 * v + slot[r];
        W[r][0] = W[r][1] = W[r][2] = 0.0;
        for (int q = 0; q < 3; ++q) D[r][q] = c_dir[slot[r]][q];
        for (int s = inc_ptr[e]; s < inc_ptr[e + 1]; ++s) {
            int t = inc[s] >> 3, l = inc[s] & 7, p = t % 6;
            double ep = eps[t];
            for (int q = 0; q < 3; ++q) W[r][q] += ep * c_wint[p][l][q];
        }
    }
    double S[3][3], G[3][3], Gp[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s1 = 0.0, s2 = 0.0, g = 0.0;
            for (int r = 0; r < k; ++r) { s1 += D[r][a] * W[r][b]; s2 += W[r][a] * D[r][b]; g += D[r][a] * D[r][b]; }
            S[a][b] = 0.5 * (s1 + s2);
            G[a][b] = g;
        }
    sym3_pinv(G, Gp);
    double lam[3], V[3][3], A[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) A[a][b] = S[a][b];
    sym3_eig(A, lam, V);
    const double mx = fmax(fabs(lam[0]), fmax(fabs(lam[1]), fabs(lam[2])));
    bool keep[3];
    for (int i = 0; i < 3; ++i) keep[i] = lam[i] > 1e-10 * mx;
    double Sp[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int i = 0; i < 3; ++i)
                if (keep[i]) s += V[a][i] * V[b][i] / lam[i];
            Sp[a][b] = s;
        }
    // QW (k x 3), then Z = QW S^+, X = W^T QW, pq
    double QW[7][3], pq = 0.0;
    for (int r = 0; r < k; ++r) {
        double q0 = 0.0, q1 = 0.0, q2 = 0.0;
        for (int c = 0; c < k; ++c) {
            double qrc = Q[28 * v + pk7(slot[r], slot[c])];
            q0 += qrc * W[c][0]; q1 += qrc * W[c][1]; q2 += qrc * W[c][2];
            double dq = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) dq += D[r][a] * Gp[a][b] * D[c][b];
            pq += ((r == c ? 1.0 : 0.0) - dq) * qrc;
        }
        QW[r][0] = q0; QW[r][1] = q1; QW[r][2] = q2;
    }
    pq /= k;
    double X[3][3], Xt[3][3], Y[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int r = 0; r < k; ++r) s += W[r][a] * QW[r][b];
            X[a][b] = s;
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) s += V[a][i] * X[a][b] * V[b][j];
            double F;
            if (keep[i] && keep[j]) F = -1.0 / (lam[i] * lam[j]);
            else if (keep[i]) F = 1.0 / (lam[i] * (lam[i] - lam[j]));
            else if (keep[j]) F = 1.0 / (lam[j] * (lam[j] - lam[i]));
            else F = 0.0;
            Xt[i][j] = F * s;
        }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) s += V[a][i] * Xt[i][j] * V[b][j];
            Y[a][b] = s;
        }
    for (int r = 0; r < k; ++r) {
        double Z[3], DY[3];
        for (int b = 0; b < 3; ++b) {
            Z[b] = QW[r][0] * Sp[0][b] + QW[r][1] * Sp[1][b] + QW[r][2] * Sp[2][b];
            DY[b] = D[r][0] * Y[0][b] + D[r][1] * Y[1][b] + D[r][2] * Y[2][b];
        }
        size_t e = 7 * v + slot[r];
        for (int s = inc_ptr[e]; s < inc_ptr[e + 1]; ++s) {
            int t = inc[s] >> 3, l = inc[s] & 7, p = t % 6;
            const double *wi = c_wint[p][l];
            double val = 0.0;
            for (int b = 0; b < 3; ++b) val += (2.0 * Z[b] + DY[b]) * wi[b];
            contrib[s] = -(val + c_wsq[p][l] * pq);
        }
    }
}

// dJ/deps_t: sum of the contributions at the incidence entries of t's six
// edges (PEC and unused slots carry none).
__global__ void tet_grad_gather_kernel(size_t ntet, const int *__restrict__ tet_edge, const unsigned char *__restrict__ pec,
                                       const int *__restrict__ inc_ptr, const int *__restrict__ inc,
                                       const double *__restrict__ contrib, double *__restrict__ grad)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntet) return;
    double g = 0.0;
    for (int l = 0; l < 6; ++l) {
        int e = tet_edge[6 * t + l];
        if (pec[e] & kPecBit) continue;
        const int code = (int)(t * 8 + l);
        for (int s = inc_ptr[e]; s < inc_ptr[e + 1]; ++s)
            if (inc[s] == code) g += contrib[s];
    }
    grad[t] = g;
}

// Block partial sums of x.y (deterministic two-pass reduction, FP64).
__global__ void dot_partial_kernel(size_t n, const double *__restrict__ x, const double *__restrict__ y, double *__restrict__ part)
{
    __shared__ double sh[256];
    double s = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        s += y ? x[i] * y[i] : x[i];   // y == nullptr: the plain sum of x
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Discrete energy of the symplectic state per node, in FP64:
// e_v = 1/2 P_v . (Minv_v P_v) + 1/2 U_v . F_v with F = K U (FP64); U, P and
// the mass blocks are the run's values widened to FP64, so this is the
// invariant of the system the run integrates.
template <class T>
__global__ void __launch_bounds__(128) tet_energy_node_kernel(size_t nnode, const T *__restrict__ minv, const T *__restrict__ P,
                                                              const T *__restrict__ U, const double *__restrict__ F,
                                                              double *__restrict__ e)
{
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nnode) return;
    double p[7], mv[28];
#pragma unroll
    for (int d = 0; d < 7; ++d) p[d] = (double)P[(size_t)d * nnode + v];
#pragma unroll
    for (int q = 0; q < 28; ++q) mv[q] = (double)minv[fpk(v, q, nnode)];
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < 7; ++d) {
        double y = 0.0;
#pragma unroll
        for (int j = 0; j < 7; ++j) {
            const int r7 = d < j ? d : j, s7 = d < j ? j : d;
            y = fma(mv[r7 * (13 - r7) / 2 + s7], p[j], y);
        }
        s = fma(0.5 * p[d], y, s);
        s = fma(0.5 * (double)U[(size_t)d * nnode + v], F[(size_t)d * nnode + v], s);
    }
    e[v] = s;
}

// y = (double)x
template <class T> __global__ void widen_kernel(size_t n, const T *__restrict__ x, double *__restrict__ y)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (double)x[i];
}

// *out = sum of the nb <= 512 partial sums, by a fixed-shape tree (one
// block of 512 threads; deterministic).
// With jp given, the coefficient pointers of the Lanczos kernels below are
// offset by 2 * (*jp): the iteration index lives on the device so that a
// captured graph of iterations can be replayed.
__global__ void __launch_bounds__(512) dot_finish_kernel(int nb, const double *__restrict__ part, double *__restrict__ out,
                                                         const int *__restrict__ jp = nullptr)
{
    __shared__ double sh[512];
    const int t = threadIdx.x;
    sh[t] = t < nb ? part[t] : 0.0;
    __syncthreads();
    for (int w = 256; w > 0; w >>= 1) {
        if (t < w) sh[t] += sh[t + w];
        __syncthreads();
    }
    if (t == 0) out[jp ? 2 * *jp : 0] = sh[0];
}

// Lanczos reductions without a finishing launch: every block writes its
// FP64 partial sum, and the block that finishes last (the one whose atomic
// ticket is gridDim.x - 1, after every block fenced its partial) adds all
// partials in block order, so the result has the same bits whichever block
// is last.  Grids are capped at kLzBlocks blocks (grid-stride loops).
constexpr int kLzBlocks = 1024;

// Block sum of s (warp butterflies, then the warps in order); every thread
// of the block must call it; the result is valid in thread 0.
__device__ __forceinline__ double block_sum(double s)
{
    __shared__ double ws[32];
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
    __syncthreads();   // ws may still be read from an earlier call
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) t += ws[w];
    return t;
}

// *out = sum over the grid of s (see above); ticket must be zero before the
// launch and is zero again after it.
__device__ __forceinline__ void grid_sum(double s, double *__restrict__ part, unsigned *__restrict__ ticket,
                                         double *__restrict__ out)
{
    __shared__ bool last;
    const double b = block_sum(s);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = b;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    double r = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) r += __ldcg(part + i);
    r = block_sum(r);
    if (threadIdx.x == 0) {
        *out = r;
        *ticket = 0u;
    }
}

// x, y *= 1 / sqrt(nrm), nrm = nrm_base[2 * *jp] with jp, else nrm_base[0];
// x32 = (float) x afterwards and kz = 0 (the FP32 buffer the next apply
// accumulates K x32 into).
__global__ void __launch_bounds__(256) scale_kernel(size_t n, double *__restrict__ x, double *__restrict__ y,
                                                    const double *__restrict__ nrm_base, const int *__restrict__ jp,
                                                    float *__restrict__ x32, float *__restrict__ kz)
{
    const double s = 1.0 / sqrt(nrm_base[jp ? 2 * *jp : 0]);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double xs = x[i] * s;
        x[i] = xs;
        y[i] *= s;
        x32[i] = (float)xs;
        kz[i] = 0.0f;
    }
}

// y = (float)x
__global__ void narrow_kernel(size_t n, const double *__restrict__ x, float *__restrict__ y)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (float)x[i];
}

// One Lanczos apply after K v was formed in FP32: per node Mw = (double)
// Kv32, w = Minv Mw (FP64 mass blocks), and *alpha = v . Mw.  With jp
// given, the device iteration index is advanced here (no kernel of this
// iteration has read it yet).
__global__ void __launch_bounds__(128) lanczos_minv_kernel(size_t nnode, const double *__restrict__ minv,
                                                           const float *__restrict__ kv32, const double *__restrict__ vcur,
                                                           double *__restrict__ Mw, double *__restrict__ w,
                                                           double *__restrict__ part, unsigned *__restrict__ ticket,
                                                           double *__restrict__ alpha, int *__restrict__ jp)
{
    if (jp && blockIdx.x == 0 && threadIdx.x == 0) *jp += 1;
    double acc = 0.0;
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nnode; v += (size_t)gridDim.x * blockDim.x) {
        double x[7], mv[28];
#pragma unroll
        for (int d = 0; d < 7; ++d) {
            const size_t f = (size_t)d * nnode + v;
            x[d] = (double)kv32[f];
            Mw[f] = x[d];
            acc += vcur[f] * x[d];
        }
        load_block<double>(minv, nnode, v, mv);
#pragma unroll
        for (int d = 0; d < 7; ++d) w[(size_t)d * nnode + v] = block_row<double>(mv, x, d);
    }
    grid_sum(acc, part, ticket, alpha);
}

// Start vector of the Lanczos iteration: per slot a value in [-0.5, 0.5)
// from the splitmix64 hash of its slot id (PEC and unused slots zero), in the
// plane layout.
__global__ void lanczos_start_kernel(size_t nslot, size_t nnode, const unsigned char *__restrict__ pec, double *__restrict__ x)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nslot) return;
    unsigned long long z = (unsigned long long)e + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    x[fslot(e, nnode)] = (pec[e] & kPecBit) ? 0.0 : (double)(z >> 11) / 9007199254740992.0 - 0.5;
}

// Lanczos three-term step on a vector and its mass image: alpha_j = *alpha
// (kept at cf[2j]), beta_j^2 at cf[2j - 1]; w -= alpha v + beta vp, Mw -=
// alpha Mv + beta Mvp (vp == nullptr: no beta term), then beta_{j+1}^2 =
// w . Mw at cf[2j + 1].  j = *jp when jp is given, else j0.
__global__ void __launch_bounds__(256) lanczos_step_kernel(size_t n, double *__restrict__ w, double *__restrict__ Mw,
                                                           const double *__restrict__ v, const double *__restrict__ Mv,
                                                           const double *__restrict__ vp, const double *__restrict__ Mvp,
                                                           const double *__restrict__ alpha, double *__restrict__ part,
                                                           unsigned *__restrict__ ticket, double *__restrict__ cf, int j0,
                                                           const int *__restrict__ jp)
{
    const int j = jp ? *jp : j0;
    const double al = *alpha, be = vp ? sqrt(cf[2 * j - 1]) : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) cf[2 * j] = al;
    double acc = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double wi = w[i] - al * v[i] - be * (vp ? vp[i] : 0.0);
        const double mi = Mw[i] - al * Mv[i] - be * (Mvp ? Mvp[i] : 0.0);
        w[i] = wi;
        Mw[i] = mi;
        acc += wi * mi;
    }
    grid_sum(acc, part, ticket, cf + 2 * j + 1);
}

// -------------------------------------------------------------- host side
double tet_wave(int kind, double f0, double t)
{
    if (kind == EMS_WAVE_RICKER) {
        double tau = t - std::sqrt(2.0) / f0;
        return (1.0 - 2.0 * M_PI * M_PI * f0 * f0 * tau * tau) * std::exp(-M_PI * M_PI * f0 * f0 * tau * tau);
    }
    double delay = t - 1.0 / f0, zeta = 2.0 * M_PI * M_PI * f0 * f0;
    return 2.0 * zeta * (2.0 * zeta * delay * delay - 1.0) * std::exp(0.0 - zeta * delay * delay) / (2.0 * zeta);
}

double stability_constant(int integrator)
{
    if (integrator != EMS_SYMP4) return 2.0;
    double x1 = 1.0 / (2.0 - std::pow(2.0, 1.0 / 3.0)), x2 = 1.0 - 2.0 * x1;
    double sub[3] = {x1, x2, x1}, lo = 0.0, hi = 4.0;
    for (int it = 0; it < 200; ++it) {
        double mid = 0.5 * (lo + hi);
        bool stable = true;
        for (int s = 1; s <= 64 && stable; ++s) {
            double w = mid * s / 64.0, A[2][2] = {{1, 0}, {0, 1}};
            for (int q = 0; q < 3; ++q) {
                double a = sub[q] * w;
                double D[2][2] = {{1, a / 2}, {0, 1}}, K[2][2] = {{1, 0}, {-a, 1}}, T1[2][2], T2[2][2], R[2][2];
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j) T1[i][j] = K[i][0] * D[0][j] + K[i][1] * D[1][j];
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j) T2[i][j] = D[i][0] * T1[0][j] + D[i][1] * T1[1][j];
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j) R[i][j] = T2[i][0] * A[0][j] + T2[i][1] * A[1][j];
                std::memcpy(A, R, sizeof(A));
            }
            if (std::fabs(A[0][0] + A[1][1]) > 2.0) stable = false;
        }
        if (stable) lo = mid; else hi = mid;
    }
    return lo;
}

struct Dipole {
    int slot[6];
    double coef[6];
    int kind;
    double f0n;   // normalised frequency
};

// One shot of a batch: a cube of cells whose nodes and tetrahedra occupy
// the ranges starting at node0 / tet0 of the concatenated mesh.
struct Shot {
    int nx, ny, nz;
    size_t node0, tet0;
};

struct TetFemSim : Sim {
    ems_tetfem_params P;
    int nx, ny, nz;                 // the first shot (single-shot handles)
    std::vector<Shot> shots;
    size_t nnode, nslot, ntet;
    bool fp64;
    double c0 = 299792458.0;
    double tscale;                  // seconds per normalised time unit (h / c0)
    double dtn = 0.0, dt_lim_n = 0.0, lambda_max = 0.0;
    std::vector<int> tet_edge_h, inc_ptr_h, inc_h, nrec_h;
    std::vector<unsigned char> pec_h;
    std::vector<double> eps_h;
    // conductivity: normalised per tetrahedron (sigma h / (c0 eps0)), the
    // per-node loss rate and its denominator, and the per-node loss factor
    // of the time loop (exp(-rho dt/2) symplectic, rho dt/2 leapfrog)
    std::vector<double> sig_h, rho_h, lden_h;
    bool has_loss = false;
    DevBuf d_damp;
    int step_block = 64;            // threads per block of tet_step_kernel (tune_launch_shape)
    bool slot_split = true;         // symplectic lossless steps by tet_slot_kernel (tune_launch_shape)
    // Until a run tunes the shape (recorded runs do not), the slot-split
    // kernel serves meshes that fit in L2, the node kernel larger ones (on
    // the 64-shot batch and the 16-shot 48^3 inversion the node kernel is
    // the faster, bandwidth-bound one).
    static constexpr size_t kSlotDefaultMaxNodes = 262144;
    bool step_tuned = false;        // the block size depends on the mesh only: tuned once per handle
    // the persistent step (tet_persist_kernel, a tuner candidate): its grid
    // barrier's counter and error word, the resident-block capacity of its
    // launch (-1: not queried yet), and whether the current run launched it
    bool persist = false;
    int persist_cap = -1;
    bool bar_used = false;
    DevBuf d_bar;
    DevBuf d_tet_edge, d_inc_ptr, d_inc, d_nrec, d_pec, d_eps, d_minv, d_U, d_P, d_Uold, d_status;
    // FP32 runs: bfloat16 compensation planes of U and then P, one
    // allocation (plane layout, updated in place; zero after a reset)
    DevBuf d_comp;
    Comp comp() const { return fp64 ? Comp{} : Comp{d_comp.as<__nv_bfloat16>()}; }
    // Workspace of the Lanczos stability limit and its captured graph of
    // three iterations, kept across set_material calls (allocating, freeing
    // and instantiating them anew cost about 0.7 ms per setup on a 32^3
    // mesh); the graph is captured again when the step block size changes.
    struct LanczosWork {
        DevBuf vb[3], mb[3], part, tickets, coef, v32, kv32, jbuf, minv;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t exec = nullptr;
        int block = 0;
        const void *reads[3] = {};   // mass blocks, slot flags and node records the graph reads
        void drop_graph()
        {
            if (exec) cudaGraphExecDestroy(exec);
            if (g) cudaGraphDestroy(g);
            exec = nullptr;
            g = nullptr;
        }
        ~LanczosWork() { drop_graph(); }
    } lz;
    std::vector<Dipole> dips;
    std::vector<std::array<int, 6>> rec_edges;
    std::vector<std::array<double, 18>> rec_w;
    DevBuf d_src_slot, d_src_coef, d_src_dip, d_src_g, d_rec_e, d_rec_w, d_rec_k, d_kslot, d_kidx, d_rz, d_tr, d_ctl;
    int nk = 0;   // distinct receiver slots
    bool ready = false;
    bool flags_dirty = false;       // pec_h gained source bits not yet on the device
    std::vector<int> rec_ks;        // receiver slots flagged in pec_h and indexed by d_kidx
    bool kidx_valid = false;        // d_kidx holds the table of rec_ks
    // recording for the adjoint: snapshots of the merged state (U, P) at the
    // start of every segment of rec_seg steps of the last run, if that run
    // started from the reset state with ckpt_nsnap > 0
    int ckpt_nsnap = 0, rec_nsteps = -1, rec_seg = 0;
    bool fresh = true;              // zero fields at t = 0
    DevBuf d_snap;
    SrcArgs rec_sa{};
    double cur_time = 0.0;          // normalised

    // cells: 3 per shot.  Every shot is an independent cube mesh; the shots
    // are concatenated so each kernel launch advances all of them.
    TetFemSim(const ems_tetfem_params *p, const std::vector<std::array<int, 3>> &cells) : Sim(Kind::TETFEM), P(*p)
    {
        EMS_CHECK_ARG(!cells.empty(), "at least one shot");
        size_t n0 = 0, t0 = 0;
        for (auto &c : cells) {
            EMS_CHECK_ARG(c[0] > 0 && c[1] > 0 && c[2] > 0, "cell counts must be positive");
            shots.push_back(Shot{c[0], c[1], c[2], n0, t0});
            n0 += (size_t)(c[0] + 1) * (c[1] + 1) * (c[2] + 1);
            t0 += 6 * (size_t)c[0] * c[1] * c[2];
        }
        nx = shots[0].nx; ny = shots[0].ny; nz = shots[0].nz;
        EMS_CHECK_ARG(P.h > 0, "h must be positive");
        EMS_CHECK_ARG(P.order == 1, "only lowest-order (order 1) Nedelec tetrahedra are implemented");
        EMS_CHECK_ARG(P.integrator == EMS_LEAPFROG || P.integrator == EMS_SYMP2 || P.integrator == EMS_SYMP4,
                      "tetrahedral integrator must be EMS_LEAPFROG, EMS_SYMP2 or EMS_SYMP4");
        EMS_CHECK_ARG(P.precision == EMS_FP64 || P.precision == EMS_FP32, "precision must be EMS_FP64 or EMS_FP32");
        EMS_CHECK_ARG(P.dt >= 0 && P.time_frequency > 0, "dt must be >= 0 and time_frequency > 0");
        if (P.cfl_fraction <= 0) P.cfl_fraction = 0.9;
        EMS_CHECK_ARG(P.cfl_fraction < 1.0, "cfl_fraction must be below 1");
        fp64 = P.precision == EMS_FP64;
        tscale = P.h / c0;
        nnode = n0;
        nslot = 7 * nnode;
        ntet = t0;
        EMS_CHECK_ARG(ntet < (size_t)1 << 28, "mesh too large for 28-bit element indices");
        EMS_CHECK_ARG(nslot < (size_t)1 << 31, "mesh too large for 32-bit slot indices");
        build_mesh();
        slot_split = nnode <= kSlotDefaultMaxNodes;
        eps_h.assign(ntet, 1.0);
        init_stream();
        upload_tables();
        upload_mesh();
    }

    size_t node(const Shot &s, int i, int j, int k) const
    {
        return s.node0 + (size_t)i + (size_t)(s.nx + 1) * ((size_t)j + (size_t)(s.ny + 1) * k);
    }
    size_t node(int i, int j, int k) const { return node(shots[0], i, j, k); }

    void build_mesh()
    {
        Shape sh[6];
        for (int p = 0; p < 6; ++p) sh[p] = make_shape(p);
        tet_edge_h.resize(6 * ntet);
        pec_h.assign(nslot, 0);
        for (const Shot &S : shots) {
            const int nx = S.nx, ny = S.ny, nz = S.nz;
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i)
                        for (int p = 0; p < 6; ++p) {
                            size_t t = S.tet0 + 6 * ((size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)) + p;
                            for (int l = 0; l < 6; ++l) {
                                const int *vm = sh[p].vert[kLoc[l][0]], *vn = sh[p].vert[kLoc[l][1]];
                                int d = dir_index(vn[0] - vm[0], vn[1] - vm[1], vn[2] - vm[2]);
                                tet_edge_h[6 * t + l] = (int)(7 * node(S, i + vm[0], j + vm[1], k + vm[2]) + d);
                            }
                        }
            const int lim[3] = {nx, ny, nz};
            for (int k = 0; k <= nz; ++k)
                for (int j = 0; j <= ny; ++j)
                    for (int i = 0; i <= nx; ++i)
                        for (int d = 0; d < 7; ++d) {
                            int a[3] = {i, j, k}, b[3] = {i + kDir[d][0], j + kDir[d][1], k + kDir[d][2]};
                            bool bad = b[0] > nx || b[1] > ny || b[2] > nz;
                            for (int q = 0; q < 3 && !bad; ++q)
                                if (a[q] == b[q] && (a[q] == 0 || a[q] == lim[q])) bad = true;
                            pec_h[7 * node(S, i, j, k) + d] = bad ? 1 : 0;
                        }
        }
        inc_ptr_h.assign(nslot + 1, 0);
        for (size_t t = 0; t < ntet; ++t)
            for (int l = 0; l < 6; ++l) inc_ptr_h[tet_edge_h[6 * t + l] + 1]++;
        for (size_t s = 0; s < nslot; ++s) inc_ptr_h[s + 1] += inc_ptr_h[s];
        inc_h.resize(6 * ntet);
        std::vector<int> fill(nslot, 0);
        for (size_t t = 0; t < ntet; ++t)
            for (int l = 0; l < 6; ++l) {
                int e = tet_edge_h[6 * t + l];
                inc_h[inc_ptr_h[e] + fill[e]++] = (int)(t * 8 + l);
            }
        // per-node records of the fused step: strides to the neighbouring
        // nodes and the mask of the neighbours that exist
        nrec_h.assign(2 * nnode, 0);
        for (const Shot &S : shots) {
            const size_t sy = (size_t)S.nx + 1, sz = sy * ((size_t)S.ny + 1);
            if (sy >= ((size_t)1 << 26) || sz > (size_t)0x7fffffff)
                throw Error{EMS_ERR_INVALID_ARGUMENT, "mesh planes too large for the node records"};
            for (int k = 0; k <= S.nz; ++k)
                for (int j = 0; j <= S.ny; ++j)
                    for (int i = 0; i <= S.nx; ++i) {
                        const size_t v = node(S, i, j, k);
                        const int mask = (i > 0 ? 1 : 0) | (i < S.nx ? 2 : 0) | (j > 0 ? 4 : 0) | (j < S.ny ? 8 : 0) |
                                         (k > 0 ? 16 : 0) | (k < S.nz ? 32 : 0);
                        nrec_h[2 * v] = step_record_x((int)sy, mask);
                        nrec_h[2 * v + 1] = (int)sz;
                    }
        }
    }

    void upload_tables()
    {
        double wi[6][6][3], ws[6][6];
        for (int p = 0; p < 6; ++p) {
            Shape s = make_shape(p);
            for (int l = 0; l < 6; ++l) {
                for (int q = 0; q < 3; ++q) wi[p][l][q] = s.wint[l][q];
                ws[p][l] = s.wsq[l];
            }
        }
        unsigned char pk[7][7];
        int q = 0;
        for (int r = 0; r < 7; ++r)
            for (int c = r; c < 7; ++c) pk[r][c] = pk[c][r] = (unsigned char)q++;
        EMS_CUDA(cudaMemcpyToSymbol(c_wint, wi, sizeof(wi)));
        EMS_CUDA(cudaMemcpyToSymbol(c_wsq, ws, sizeof(ws)));
        EMS_CUDA(cudaMemcpyToSymbol(c_dir, kDir, sizeof(kDir)));
        EMS_CUDA(cudaMemcpyToSymbol(c_pack, pk, sizeof(pk)));
    }

    template <class V> void up(DevBuf &d, const std::vector<V> &v)
    {
        d.ensure(v.size() * sizeof(V));
        EMS_CUDA(cudaMemcpyAsync(d.p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, stream));
    }

    void upload_mesh()
    {
        up(d_tet_edge, tet_edge_h);
        up(d_inc_ptr, inc_ptr_h);
        up(d_inc, inc_h);
        up(d_nrec, nrec_h);
        up(d_pec, pec_h);
        size_t w = fp64 ? 8 : 4;
        d_U.alloc(nslot * w); d_U.zero(stream);
        d_P.alloc(nslot * w); d_P.zero(stream);
        d_Uold.alloc(nslot * w); d_Uold.zero(stream);
        if (!fp64) {
            d_comp.alloc(nslot * 2);
            d_comp.zero(stream);
        }
        d_minv.alloc(28 * nnode * w);
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    void set_material(const double *eps_r, const double *sigma)
    {
        EMS_CHECK_ARG(eps_r != nullptr, "eps_r required");
        for (size_t t = 0; t < ntet; ++t) EMS_CHECK_ARG(std::isfinite(eps_r[t]) && eps_r[t] > 0, "eps_r must be positive");
        if (sigma)
            for (size_t t = 0; t < ntet; ++t) EMS_CHECK_ARG(std::isfinite(sigma[t]) && sigma[t] >= 0, "sigma must be >= 0");
        eps_h.assign(eps_r, eps_r + ntet);
        sig_h.assign(ntet, 0.0);
        has_loss = false;
        if (sigma)
            for (size_t t = 0; t < ntet; ++t) {
                sig_h[t] = sigma[t] * tscale / kEps0;
                has_loss = has_loss || sigma[t] > 0;
            }
        ready = false;
        rec_nsteps = -1;   // the recorded run used the old mass blocks
    }

    void set_checkpoints(int nsnap)
    {
        EMS_CHECK_ARG(nsnap >= 0, "snapshot count must be >= 0");
        if (nsnap > 0 && P.integrator == EMS_LEAPFROG)
            throw Error{EMS_ERR_UNSUPPORTED, "the adjoint is implemented for the symplectic integrators only"};
        ckpt_nsnap = nsnap;
        if (nsnap == 0) { rec_nsteps = -1; d_snap.release(); }
    }

    // FP64 mass-inverse setup on the GPU, then the stability limit (Lanczos,
    // lambda_max_lanczos) and the time step.
    void setup()
    {
        if (d_eps.bytes == eps_h.size() * sizeof(double))   // same size: no reallocation
            EMS_CUDA(cudaMemcpyAsync(d_eps.p, eps_h.data(), d_eps.bytes, cudaMemcpyHostToDevice, stream));
        else
            up(d_eps, eps_h);
        if (!d_status.p) d_status.alloc(sizeof(int));
        if (!d_bar.p) {
            d_bar.alloc(16);
            d_bar.zero(stream);
        }
        d_status.zero(stream);
        // FP64 packed blocks for the stability limit: the run's own array in
        // FP64 runs, a copy kept with the Lanczos workspace in FP32 runs
        if (!fp64 && !lz.minv.p) lz.minv.alloc(28 * nnode * 8);
        const DevBuf &minv_d = fp64 ? d_minv : lz.minv;
        unsigned nb = (unsigned)((nnode + 127) / 128);
        tet_minv_setup_kernel<<<nb, 128, 0, stream>>>(nnode, d_pec.as<unsigned char>(), d_inc_ptr.as<int>(), d_inc.as<int>(),
                                                      d_eps.as<double>(), minv_d.as<double>(),
                                                      fp64 ? nullptr : d_minv.as<float>(), d_status.as<int>());
        EMS_CUDA(cudaGetLastError());
        int bad = 0;
        EMS_CUDA(cudaMemcpyAsync(&bad, d_status.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        if (bad) throw Error{EMS_ERR_NOT_FINITE, "mass block is not positive definite"};
        if (P.dt > 0) {
            dtn = P.dt / tscale;
            lambda_max = lambda_max_lanczos(minv_d, 400);
            dt_lim_n = stability_constant(P.integrator) / std::sqrt(lambda_max);
        } else {
            lambda_max = lambda_max_lanczos(minv_d, 400);
            dt_lim_n = stability_constant(P.integrator) / std::sqrt(lambda_max);
            dtn = P.cfl_fraction * dt_lim_n;
        }
        if (dtn >= dt_lim_n) throw Error{EMS_ERR_INVALID_ARGUMENT, "time step exceeds the stability limit of the integrator"};
        loss_setup();
        force_launch_shape();
        ready = true;
    }

    // Launch shape of the fused step: the node kernel at four block sizes
    // (32, 64, 128, 256 threads), the slot-split kernel, or the persistent
    // step (the slot-split step for a graph's 12 steps in one cooperative
    // launch with grid barriers between substeps; symplectic lossless runs
    // whose grid fits in one wave, else its runs take the slot-split
    // kernel).  It depends on the mesh, not the material, and changes no
    // result, so it is chosen once per handle inside its first unrecorded
    // run of at least 156 steps (symplectic or leapfrog): each available
    // candidate advances 12 real steps of that run from a CUDA graph, as the
    // loop runs them, twice over, and the fastest is kept for the rest of
    // the run and later ones.  (Timed on idle steps outside a run, the
    // candidates ranked differently from the loop.)  Before that the
    // slot-split kernel runs on meshes of up to kSlotDefaultMaxNodes nodes
    // and the 64-thread node kernel on larger ones.  The environment
    // variable EMS_TET_STEP_BLOCK (32, 64, 128, 256, slot or persist) forces
    // one; EMS_TET_TUNE_LOG prints the candidates' times to stderr.
    static constexpr int kShapes = 6, kTuneRounds = 2, kShapeSlot = 4, kShapePersist = 5;
    void set_shape(int ci)
    {
        slot_split = ci >= kShapeSlot;
        persist = ci == kShapePersist;
        step_block = kStepBlocks[ci < 4 ? ci : 0];
    }
    void force_launch_shape()
    {
        const char *env = std::getenv("EMS_TET_STEP_BLOCK");
        if (step_tuned || !env) return;
        step_tuned = true;
        if (std::strcmp(env, "slot") == 0) { set_shape(kShapeSlot); return; }
        if (std::strcmp(env, "persist") == 0) { set_shape(kShapePersist); return; }
        const int b = std::atoi(env);
        for (int c = 0; c < 4; ++c)
            if (kStepBlocks[c] == b) { set_shape(c); return; }
        throw Error{EMS_ERR_INVALID_ARGUMENT, "EMS_TET_STEP_BLOCK must be 32, 64, 128, 256, slot or persist"};
    }

    // Blocks of the persistent step that are resident at once on this
    // device (its cooperative launch needs the whole grid resident).
    int persist_capacity()
    {
        if (persist_cap >= 0) return persist_cap;
        int dev = 0, nsm = 0, nbps = 0;
        EMS_CUDA(cudaGetDevice(&dev));
        EMS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        if (fp64) EMS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbps, tet_persist_kernel<double, 0>, kSlotThreads, 0));
        else EMS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbps, tet_persist_kernel<float, 1>, kSlotThreads, 0));
        persist_cap = nbps * nsm;
        return persist_cap;
    }
    // Grid of the persistent step: the receiver-sampling blocks (eight
    // lanes per receiver), then one block per 32 nodes.
    unsigned persist_grid(bool sampling) const
    {
        const int nsb = sampling && nobs > 0 ? (nobs + kSlotThreads / 8 - 1) / (kSlotThreads / 8) : 0;
        return (unsigned)nsb + (unsigned)((nnode + kSlotNodes - 1) / kSlotNodes);
    }
    bool can_persist(bool symp)
    {
        return symp && !has_loss && persist_grid(true) <= (unsigned)persist_capacity();
    }
    // The barrier of a persistent launch: the whole grid arrives, a wait
    // gives up after one second.  EMS_TET_BARRIER_PROBE=1 makes the barrier
    // expect one block more than the grid holds, a count that is never
    // reached, so every wait runs out (after 20 ms) and the run returns
    // EMS_ERR_DEVICE_TIMEOUT: the test of that status path.
    GridBarrier barrier_args(unsigned grid) const
    {
        GridBarrier b{d_bar.as<unsigned>(), d_bar.as<int>() + 1, grid, 1000000000ull};
        const char *probe = std::getenv("EMS_TET_BARRIER_PROBE");
        if (probe && std::strcmp(probe, "1") == 0) {
            b.expected = grid + 1;
            b.limit_ns = 20000000ull;
        }
        return b;
    }

    // Conductivity as a per-node loss rate: rho_v = sum sigma_T w / sum
    // eps_T w over the incidences (T, l) of the node's live slots, w =
    // |w_l|^2 integral (the weights of the mass block's alpha term), so
    // M_sigma,v = rho_v M_eps,v and the loss term of the momentum equation
    // is rho_v P.  The symplectic loop applies its flow exp(-rho dt/2) on
    // each side of the middle kick (a time-symmetric composition, second
    // order when sigma != 0); leapfrog takes the centred loss term.  Host
    // FP64, O(ntet).
    void loss_setup()
    {
        rho_h.assign(nnode, 0.0);
        lden_h.assign(nnode, 0.0);
        if (!has_loss) { d_damp.release(); return; }
        double wsq[6][6];
        for (int p = 0; p < 6; ++p) {
            const Shape sh = make_shape(p);
            for (int l = 0; l < 6; ++l) wsq[p][l] = sh.wsq[l];
        }
        const bool symp = schedule().symp;
        std::vector<double> dmp(nnode);
        for (size_t v = 0; v < nnode; ++v) {
            double num = 0.0, den = 0.0;
            for (int d = 0; d < 7; ++d) {
                const size_t e = 7 * v + d;
                if (pec_h[e] & kPecBit) continue;
                for (int q = inc_ptr_h[e]; q < inc_ptr_h[e + 1]; ++q) {
                    const int t = inc_h[q] >> 3, l = inc_h[q] & 7, p = t % 6;
                    num += sig_h[t] * wsq[p][l];
                    den += eps_h[t] * wsq[p][l];
                }
            }
            rho_h[v] = den > 0.0 ? num / den : 0.0;
            lden_h[v] = den;
            dmp[v] = symp ? std::exp(-0.5 * dtn * rho_h[v]) : 0.5 * dtn * rho_h[v];
        }
        if (fp64) {
            up(d_damp, dmp);
        } else {
            std::vector<float> f(dmp.begin(), dmp.end());
            up(d_damp, f);
        }
    }

    // *out = x.y on the device (deterministic: block partials, then their
    // sum in order)
    void dot(const DevBuf &x, const DevBuf &y, DevBuf &part, double *out, const int *jp = nullptr)
    {
        const int nb = 512;
        dot_partial_kernel<<<nb, 256, 0, stream>>>(nslot, x.as<double>(), y.as<double>(), part.as<double>());
        dot_finish_kernel<<<1, 512, 0, stream>>>(nb, part.as<double>(), out, jp);
    }

    // z = K x in FP64 through the force-only fused step (P = z = 0, a = -1)
    void applyK64(const DevBuf &x, DevBuf &z)
    {
        z.zero(stream);
        const unsigned nbv = (unsigned)((nnode + step_block - 1) / step_block);
        tet_step_kernel<double, 0, 0><<<nbv, step_block, 0, stream>>>(nnode, d_nrec.as<int2>(), d_pec.as<unsigned char>(), nullptr,
                                                               z.as<double>(), x.as<double>(), nullptr, nullptr, -1.0, 0.0,
                                                               SrcArgs{}, nullptr, nullptr, nullptr, nullptr, RecArgs<double>{}, Comp{});
    }

    // Mz = K x formed in FP32 from x32 (accumulated into kv32, which must be
    // zero) and z = Minv Mz in FP64, with *alpha = vcur . Mz: one Lanczos
    // apply.  K x in FP64 is the same fused step, but GB300
    // issues FP64 at a small fraction of its FP32 rate and the FP64 step took
    // about 50 us per apply on a 32^3 mesh.
    void applyMinvK32(const DevBuf &x32, DevBuf &kv32, const DevBuf &minv_d, const DevBuf &vcur, DevBuf &Mz, DevBuf &z,
                      DevBuf &part, unsigned *ticket, double *alpha, int *jp, int max_blocks)
    {
        const unsigned nbv = (unsigned)((nnode + step_block - 1) / step_block);
        tet_step_kernel<float, 0, 0><<<nbv, step_block, 0, stream>>>(nnode, d_nrec.as<int2>(), d_pec.as<unsigned char>(), nullptr,
                                                              kv32.as<float>(), x32.as<float>(), nullptr, nullptr, -1.0f, 0.0f,
                                                              SrcArgs{}, nullptr, nullptr, nullptr, nullptr, RecArgs<float>{}, Comp{});
        const int nb = (int)std::min<size_t>((nnode + 127) / 128, max_blocks);
        lanczos_minv_kernel<<<nb, 128, 0, stream>>>(nnode, minv_d.as<double>(), kv32.as<float>(), vcur.as<double>(),
                                                    Mz.as<double>(), z.as<double>(), part.as<double>(), ticket, alpha, jp);
    }

    // Largest eigenvalue of Minv K by Lanczos in the M inner product.  Minv K
    // is self-adjoint there, and every Lanczos vector v travels with its mass
    // image Mv: K v is the mass image of w = Minv K v, so <v, w>_M = v.K v and
    // <w, w>_M = w.(M w) need no M.  The start pair is x = Minv K x0, Mx =
    // K x0.  K v is formed in FP32 by the fused step (applyMinvK32), Minv
    // K v, the dot products and the recurrence in FP64; the largest Ritz
    // value then agrees with an all-FP64 iteration to about 1e-6 relative.
    // The tridiagonal coefficients stay on the device; every 6 steps
    // the largest eigenvalue of the tridiagonal matrix (Sturm bisection) is
    // checked and the iteration stops once it changes by less than 1e-8
    // relative (Ritz values approach it from below, and the time step is a
    // fraction of the limit: 1e-8 is far below any effect on it).
    // Without reorthogonalisation converged Ritz values repeat, which does
    // not move the largest one.
    double lambda_max_lanczos(const DevBuf &minv_d, int max_iters)
    {
        LanczosWork &w = lz;
        if (!w.v32.p) {
            for (int q = 0; q < 3; ++q) { w.vb[q].alloc(nslot * 8); w.mb[q].alloc(nslot * 8); }
            w.v32.alloc(nslot * 4);    // FP32 copy of the vector K is applied to
            w.kv32.alloc(nslot * 4);   // K v in FP32 (zeroed by each scale launch for the next apply)
            w.part.alloc(kLzBlocks * 8);   // block partials of the reductions
            w.tickets.alloc(2 * sizeof(unsigned));
            w.tickets.zero(stream);
            // alpha_j at [2j], beta_{j+1}^2 at [2j+1]; scratch at 2 max_iters + 10 (start norm) and + 11 (alpha)
            w.coef.alloc(2 * (max_iters + 6) * 8);
            w.jbuf.alloc(sizeof(int));
        }
        int nsm = 0;
        EMS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0));
        unsigned *tk = w.tickets.as<unsigned>();
        const unsigned nbs = (unsigned)((nslot + 255) / 256);
        // the reducing launches: at most two blocks per SM (grid-stride), so
        // that few blocks queue on the atomic ticket of the last-block sum
        const int nbl = (int)std::min<size_t>(nbs, std::min(kLzBlocks, 2 * std::max(nsm, 1)));
        double *cf = w.coef.as<double>(), *nrm0 = cf + 2 * max_iters + 10, *alpha = cf + 2 * max_iters + 11;
        DevBuf *vb = w.vb, *mb = w.mb;
        // start pair (v1, Mv1) = (Minv K x0, K x0) / |.|_M, in buffers 1
        lanczos_start_kernel<<<nbs, 256, 0, stream>>>(nslot, nnode, d_pec.as<unsigned char>(), vb[0].as<double>());
        narrow_kernel<<<nbs, 256, 0, stream>>>(nslot, vb[0].as<double>(), w.v32.as<float>());
        w.kv32.zero(stream);
        applyMinvK32(w.v32, w.kv32, minv_d, vb[0], mb[1], vb[1], w.part, tk, alpha, nullptr, nbl);
        dot_partial_kernel<<<512, 256, 0, stream>>>(nslot, vb[1].as<double>(), mb[1].as<double>(), w.part.as<double>());
        dot_finish_kernel<<<1, 512, 0, stream>>>(512, w.part.as<double>(), nrm0);
        scale_kernel<<<nbl, 256, 0, stream>>>(nslot, vb[1].as<double>(), mb[1].as<double>(), nrm0, nullptr, w.v32.as<float>(),
                                              w.kv32.as<float>());
        int prev = -1, cur = 1, nxt = 2;
        // one iteration: apply (+ alpha), three-term step (+ beta^2),
        // normalisation; jp == nullptr: host index jj, else the device index
        // (advanced by the apply)
        auto iteration = [&](int jj, int *jp) {
            applyMinvK32(w.v32, w.kv32, minv_d, vb[cur], mb[nxt], vb[nxt], w.part, tk, alpha, jp, nbl);
            lanczos_step_kernel<<<nbl, 256, 0, stream>>>(nslot, vb[nxt].as<double>(), mb[nxt].as<double>(), vb[cur].as<double>(),
                                                         mb[cur].as<double>(), prev >= 0 ? vb[prev].as<double>() : nullptr,
                                                         prev >= 0 ? mb[prev].as<double>() : nullptr, alpha,
                                                         w.part.as<double>(), tk + 1, cf, jj, jp);
            scale_kernel<<<nbl, 256, 0, stream>>>(nslot, vb[nxt].as<double>(), mb[nxt].as<double>(),
                                                  jp ? cf + 1 : cf + 2 * jj + 1, jp, w.v32.as<float>(), w.kv32.as<float>());
            const int t = prev < 0 ? 0 : prev;
            prev = cur; cur = nxt; nxt = t;
        };
        iteration(0, nullptr);
        // iterations 1, 2, 3, ...: after the first, the three buffers rotate
        // with period 3, so one captured graph of three iterations (the
        // coefficient index on the device, advanced to 1 by the first
        // replayed apply) is replayed; the largest Ritz value is checked
        // every six iterations
        EMS_CUDA(cudaMemsetAsync(w.jbuf.p, 0, sizeof(int), stream));
        const void *reads[3] = {minv_d.p, d_pec.p, d_nrec.p};
        if (!w.exec || w.block != step_block || !std::equal(reads, reads + 3, w.reads)) {
            w.drop_graph();
            EMS_CUDA(cudaStreamSynchronize(stream));
            EMS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            for (int q = 0; q < 3; ++q) iteration(0, w.jbuf.as<int>());
            cudaError_t ce = cudaStreamEndCapture(stream, &w.g);
            if (ce != cudaSuccess) throw Error{EMS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce)};
            ce = cudaGraphInstantiate(&w.exec, w.g, 0);
            if (ce != cudaSuccess) {
                w.exec = nullptr;
                throw Error{EMS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce)};
            }
            w.block = step_block;
            std::copy(reads, reads + 3, w.reads);
        }
        std::vector<double> h;
        double lam = 0.0, lam_old = -1.0;
        for (int done = 1, rep = 1; done < max_iters; ++rep) {
            EMS_CUDA(cudaGraphLaunch(w.exec, stream));
            done += 3;
            if (rep % 2 == 0 || done >= max_iters) {
                h.resize(2 * done);
                EMS_CUDA(cudaMemcpyAsync(h.data(), cf, h.size() * 8, cudaMemcpyDeviceToHost, stream));
                EMS_CUDA(cudaStreamSynchronize(stream));
                lam = tridiag_max_eig(h, done);
                const bool breakdown = !(h[2 * done - 1] > 1e-300);
                if (breakdown || std::fabs(lam - lam_old) <= 1e-8 * lam) break;
                lam_old = lam;
            }
        }
        EMS_CUDA(cudaGetLastError());
        return lam;
    }

    // Largest eigenvalue of the symmetric tridiagonal matrix with diagonal
    // h[0], h[2], ... and squared off-diagonals h[1], h[3], ... (m x m), by
    // bisection on the Sturm count of eigenvalues below x.
    static double tridiag_max_eig(const std::vector<double> &h, int m)
    {
        double lo = 1e300, hi = -1e300;
        for (int i = 0; i < m; ++i) {
            const double r = (i > 0 ? std::sqrt(h[2 * i - 1]) : 0.0) + (i + 1 < m ? std::sqrt(h[2 * i + 1]) : 0.0);
            lo = std::min(lo, h[2 * i] - r);
            hi = std::max(hi, h[2 * i] + r);
        }
        auto below = [&](double x) {   // eigenvalues < x
            int c = 0;
            double d = 1.0;
            for (int i = 0; i < m; ++i) {
                d = h[2 * i] - x - (i > 0 ? h[2 * i - 1] / d : 0.0);
                if (d == 0.0) d = -1e-300;
                if (d < 0.0) ++c;
            }
            return c;
        };
        for (int it = 0; it < 200 && hi - lo > 1e-15 * std::fabs(hi); ++it) {
            const double mid = 0.5 * (lo + hi);
            if (below(mid) >= m) hi = mid; else lo = mid;
        }
        return hi;
    }

    void locate(const Shot &S, const double xn[3], double w[6][3], int edges[6]) const
    {
        int cell[3], lim[3] = {S.nx, S.ny, S.nz};
        double s[3];
        for (int q = 0; q < 3; ++q) {
            int c = (int)std::floor(xn[q]);
            c = std::max(0, std::min(c, lim[q] - 1));
            cell[q] = c;
            s[q] = xn[q] - c;
        }
        int ax[3] = {0, 1, 2};
        for (int a = 1; a < 3; ++a)
            for (int b = a; b > 0 && s[ax[b - 1]] < s[ax[b]]; --b) std::swap(ax[b], ax[b - 1]);
        int p = 0;
        for (; p < 6; ++p)
            if (kPerm[p][0] == ax[0] && kPerm[p][1] == ax[1] && kPerm[p][2] == ax[2]) break;
        double lam[4] = {1.0 - s[ax[0]], s[ax[0]] - s[ax[1]], s[ax[1]] - s[ax[2]], s[ax[2]]};
        Shape sh = make_shape(p);
        for (int l = 0; l < 6; ++l) {
            int a = kLoc[l][0], b = kLoc[l][1];
            for (int q = 0; q < 3; ++q) w[l][q] = lam[a] * sh.grad[b][q] - lam[b] * sh.grad[a][q];
            const int *vm = sh.vert[a], *vn = sh.vert[b];
            int d = dir_index(vn[0] - vm[0], vn[1] - vm[1], vn[2] - vm[2]);
            edges[l] = (int)(7 * node(S, cell[0] + vm[0], cell[1] + vm[1], cell[2] + vm[2]) + d);
        }
    }

    // Substeps of one time step in normalised units: kick lengths sub[q],
    // source-time offsets off[q], merged drift lengths c[q] (the second half
    // of substep q plus the first half of the next one) and the first half
    // drift hfirst.
    struct Schedule {
        bool symp;
        int nsub;
        double sub[3], off[3], c[3], hfirst;
    };
    Schedule schedule() const
    {
        Schedule s{};
        s.symp = P.integrator != EMS_LEAPFROG;
        s.nsub = P.integrator == EMS_SYMP4 ? 3 : 1;
        s.sub[0] = dtn;
        if (s.nsub == 3) {
            const double x1 = 1.0 / (2.0 - std::pow(2.0, 1.0 / 3.0)), x2 = 1.0 - 2.0 * x1;
            s.sub[0] = x1 * dtn; s.sub[1] = x2 * dtn; s.sub[2] = x1 * dtn;
            s.off[1] = x1 * dtn; s.off[2] = (x1 + x2) * dtn;
        }
        for (int q = 0; q < s.nsub; ++q) s.c[q] = 0.5 * (s.sub[q] + s.sub[q + 1 < s.nsub ? q + 1 : 0]);
        s.hfirst = 0.5 * s.sub[0];
        return s;
    }

    // One substep (tet_step_kernel): MODE 0 (symplectic) P -= a (K Uin - f);
    // Uout = Uin + c Minv P (zout = Minv P), or MODE 1 (leapfrog) Uout =
    // 2 Uin - Uold - c Minv (K Uin - f); DAMP selects the lossy forms (the
    // middle kick, its adjoint, the lossy leapfrog).  Uout is a different
    // buffer from Uin.  Returns the number of launches.
    // cm: the compensation planes of Uin/Uout and Pio (FP32 symplectic
    // steps; empty for FP64 and leapfrog).
    template <class T, int MODE, int DAMP = 0>
    int substep(const T *Uin, T *Uout, T *Pio, const T *Uold, T a, T c, const SrcArgs &sa, T *zout, T *ppre = nullptr,
                T *pmid = nullptr, const RecArgs<T> &rec = RecArgs<T>{}, Comp cm = Comp{})
    {
        if (Uin == Uout) throw Error{EMS_ERR_STATE, "fused step needs separate input and output fields"};
        if constexpr (MODE == 0 && DAMP == 0) {
            if (slot_split) {
                // rec.nsb leading blocks sample the receivers when this launch does
                const unsigned nbs = (unsigned)((nnode + kSlotNodes - 1) / kSlotNodes) + (unsigned)rec.nsb;
                const dim3 blk(kSlotNodes, 7);
                auto go = [&](auto kern) {
                    kern<<<nbs, blk, 0, stream>>>(nnode, d_nrec.as<int2>(), d_pec.as<unsigned char>(), d_minv.as<T>(), Pio,
                                                  Uin, Uout, a, c, sa, zout, rec, cm);
                    return 1;
                };
                const bool comp32 = std::is_same<T, float>::value && cm.p;
                if (rec.rz_out) return comp32 ? go(tet_slot_kernel<T, 1, 1>) : go(tet_slot_kernel<T, 1, 0>);
                return comp32 ? go(tet_slot_kernel<T, 0, 1>) : go(tet_slot_kernel<T, 0, 0>);
            }
        }
        // rec.nsb leading blocks sample the receivers when this launch does
        const unsigned nbv = (unsigned)((nnode + step_block - 1) / step_block) + (unsigned)rec.nsb;
        const T *dm = DAMP ? d_damp.as<T>() : nullptr;
        auto go = [&](auto kern) {
            kern<<<nbv, step_block, 0, stream>>>(nnode, d_nrec.as<int2>(), d_pec.as<unsigned char>(), d_minv.as<T>(), Pio, Uin,
                                                 Uout, Uold, a, c, sa, zout, dm, ppre, pmid, rec, cm);
            return 1;
        };
        if constexpr (MODE == 0 && std::is_same<T, float>::value) {
            if (cm.p) {
                if constexpr (DAMP != 2)
                    if (rec.rz_out) return go(tet_step_kernel<T, MODE, DAMP, 1, 1>);
                return go(tet_step_kernel<T, MODE, DAMP, 0, 1>);
            }
        }
        if constexpr (MODE == 0 && DAMP != 2)
            if (rec.rz_out) return go(tet_step_kernel<T, MODE, DAMP, 1>);
        return go(tet_step_kernel<T, MODE, DAMP>);
    }

    // The loop's step with a = c = 0 (P, U and their compensation keep their
    // values; U is copied into the other buffer of the pair), for the
    // launch-shape tuner and the dominant-kernel timing.  odd swaps the pair.
    void idle_step(unsigned nbv, int odd)
    {
        auto body = [&](auto tag) {
            using T = decltype(tag);
            T *a = d_U.as<T>(), *b = d_Uold.as<T>();
            if (odd) std::swap(a, b);
            const Comp cm = comp();
            if (slot_split) {
                const unsigned nbs = (unsigned)((nnode + kSlotNodes - 1) / kSlotNodes);
                const dim3 blk(kSlotNodes, 7);
                if (cm.p)
                    tet_slot_kernel<T, 0, std::is_same<T, float>::value><<<nbs, blk, 0, stream>>>(
                        nnode, d_nrec.as<int2>(), d_pec.as<unsigned char>(), d_minv.as<T>(), d_P.as<T>(), a, b, T(0), T(0),
                        SrcArgs{}, nullptr, RecArgs<T>{}, cm);
                else
                    tet_slot_kernel<T, 0, 0><<<nbs, blk, 0, stream>>>(nnode, d_nrec.as<int2>(), d_pec.as<unsigned char>(),
                                                                     d_minv.as<T>(), d_P.as<T>(), a, b, T(0), T(0), SrcArgs{},
                                                                     nullptr, RecArgs<T>{}, Comp{});
                return;
            }
            if (cm.p)
                tet_step_kernel<T, 0, 0, 0, std::is_same<T, float>::value><<<nbv, step_block, 0, stream>>>(
                    nnode, d_nrec.as<int2>(), d_pec.as<unsigned char>(), d_minv.as<T>(), d_P.as<T>(), a, b, nullptr, T(0), T(0),
                    SrcArgs{}, nullptr, nullptr, nullptr, nullptr, RecArgs<T>{}, cm);
            else
                tet_step_kernel<T, 0, 0><<<nbv, step_block, 0, stream>>>(nnode, d_nrec.as<int2>(), d_pec.as<unsigned char>(),
                                                                         d_minv.as<T>(), d_P.as<T>(), a, b, nullptr, T(0), T(0),
                                                                         SrcArgs{}, nullptr, nullptr, nullptr, nullptr,
                                                                         RecArgs<T>{}, Comp{});
        };
        if (fp64) body(double()); else body(float());
    }

    // One time step: receivers (and the step counter), then for the
    // symplectic steps one fused kick + drift per substep with the drifts
    // merged (the last one also carries the first half drift of the next
    // step), P in place and U from Uc into Uo with (Uc, Uo) swapped after
    // every substep; for leapfrog one update into Uo and the ring rotation
    // (Uc, Pc, Uo) <- (Uo, Uc, Pc).  zout (symplectic only): Minv P of
    // substep q goes to zout + q * nslot.  Returns the number of launches.
    // With losses the middle kick of a symplectic step is the lossy one;
    // prec (recorded runs) receives P before its first loss factor and
    // after the kick, at prec and prec + nslot.
    // Receiver arguments of substep q of a step with counter parity par:
    // the first launch samples (and advances the counter), the last one of
    // a symplectic step keeps Minv P of the receiver slots for the next.
    // sample == false (segment recomputes of the adjoint, whose traces were
    // recorded): no sampling blocks and no Minv P kept at the receiver slots,
    // only the step counter advance the source terms read.
    template <class T> RecArgs<T> rec_args(const Schedule &sc, int q, int par, bool sample = true)
    {
        RecArgs<T> r{};
        const int nrz = std::max(nk, 1);
        if (q == 0) {
            r.nrec = sample ? nobs : 0;
            // the first launch runs the slot-split kernel unless it is the lossy middle kick or leapfrog
            const bool slot0 = slot_split && sc.symp && !(has_loss && sc.nsub / 2 == 0);
            const int per = (slot0 ? kSlotThreads : step_block) / 8;   // eight lanes per receiver
            r.nsb = sample && nobs > 0 ? (nobs + per - 1) / per : 0;
            r.adv = 1;
        }
        r.edges = d_rec_e.as<int>();
        r.rk = d_rec_k.as<int>();
        r.w = d_rec_w.as<double>();
        r.rz_in = d_rz.as<T>() + (size_t)par * nrz;
        r.unmerge = sc.symp ? (T)sc.hfirst : T(0);
        r.tr = d_tr.as<double>();
        r.nsamp = nsamp;
        r.tf = P.time_frequency;
        r.nk = nk;
        r.kslot = d_kslot.as<int>();
        r.kidx = d_kidx.as<int>();
        if (sample && sc.symp && q == sc.nsub - 1 && nk > 0) r.rz_out = d_rz.as<T>() + (size_t)(1 - par) * nrz;
        r.ctl = d_ctl.as<int>();
        r.par = par;
        return r;
    }

    // One time step n (counter parity par = n % 2).  Returns the number of
    // launches.
    template <class T>
    int enqueue_step(T *&Uc, T *&Pc, T *&Uo, const Schedule &sc, const SrcArgs &sa0, T *zout, int par, T *prec = nullptr,
                     bool sample = true, Comp cm = Comp{})
    {
        int nl = 0;
        if (sc.symp) {
            for (int q = 0; q < sc.nsub; ++q) {
                SrcArgs sa = sa0;
                sa.q = q;
                sa.par = par;
                const RecArgs<T> ra = rec_args<T>(sc, q, par, sample);
                T *z = zout ? zout + (size_t)q * nslot : nullptr;
                if (has_loss && q == sc.nsub / 2)
                    nl += substep<T, 0, 1>(Uc, Uo, Pc, nullptr, (T)sc.sub[q], (T)sc.c[q], sa, z, prec,
                                           prec ? prec + nslot : nullptr, ra, cm);
                else
                    nl += substep<T, 0>(Uc, Uo, Pc, nullptr, (T)sc.sub[q], (T)sc.c[q], sa, z, nullptr, nullptr, ra, cm);
                std::swap(Uc, Uo);
            }
        } else {
            SrcArgs sa = sa0;
            sa.par = par;
            const RecArgs<T> ra = rec_args<T>(sc, 0, par);
            if (has_loss)
                nl += substep<T, 1, 1>(Uc, Uo, nullptr, Pc, T(0), (T)(dtn * dtn), sa, nullptr, nullptr, nullptr, ra);
            else
                nl += substep<T, 1>(Uc, Uo, nullptr, Pc, T(0), (T)(dtn * dtn), sa, nullptr, nullptr, nullptr, ra);
            T *tmp = Pc; Pc = Uc; Uc = Uo; Uo = tmp;
        }
        return nl;
    }

    // nst symplectic lossless steps from step parity par0 in one
    // cooperative launch of tet_persist_kernel (U from Uc, the pair swapped
    // when the launch runs an odd number of substeps).  idle: a = c = 0, no
    // sources, receivers or counter (the dominant-kernel timing).  Returns 1.
    template <class T>
    int persist_launch(int nst, T *&Uc, T *&Pc, T *&Uo, const Schedule &sc, const SrcArgs &sa, int par0, Comp cm,
                       bool idle = false)
    {
        PersistArgs<T> pa{};
        pa.U[0] = Uc;
        pa.U[1] = Uo;
        pa.P = Pc;
        pa.cp = cm.p;
        for (int q = 0; q < sc.nsub; ++q) {
            pa.a[q] = idle ? T(0) : (T)sc.sub[q];
            pa.c[q] = idle ? T(0) : (T)sc.c[q];
        }
        pa.nsub = sc.nsub;
        pa.nsteps = nst;
        pa.par0 = par0;
        pa.rz = d_rz.as<T>();
        pa.nrz = std::max(nk, 1);
        pa.keep_rz = !idle && nk > 0;
        const RecArgs<T> ra = idle ? RecArgs<T>{} : rec_args<T>(sc, 0, par0, true);
        const unsigned grid = persist_grid(!idle);
        pa.bar = barrier_args(grid);
        const SrcArgs src = idle ? SrcArgs{} : sa;
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(kSlotNodes, 7);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        const int2 *nr = d_nrec.as<int2>();
        const unsigned char *pc = d_pec.as<unsigned char>();
        const T *mv = d_minv.as<T>();
        if constexpr (std::is_same<T, float>::value) {
            if (cm.p) EMS_CUDA(cudaLaunchKernelEx(&cfg, tet_persist_kernel<T, 1>, nnode, nr, pc, mv, pa, src, ra));
            else EMS_CUDA(cudaLaunchKernelEx(&cfg, tet_persist_kernel<T, 0>, nnode, nr, pc, mv, pa, src, ra));
        } else {
            EMS_CUDA(cudaLaunchKernelEx(&cfg, tet_persist_kernel<T, 0>, nnode, nr, pc, mv, pa, src, ra));
        }
        bar_used = true;
        if ((nst * sc.nsub) & 1) std::swap(Uc, Uo);
        return 1;
    }

    // nst steps of the time loop from step parity par0: one persistent
    // launch in that launch shape, else enqueue_step per step.  Returns the
    // number of launches.
    template <class T>
    int enqueue_steps(int nst, T *&Uc, T *&Pc, T *&Uo, const Schedule &sc, const SrcArgs &sa, int par0, Comp cm)
    {
        if (nst <= 0) return 0;
        if (persist && can_persist(sc.symp)) return persist_launch<T>(nst, Uc, Pc, Uo, sc, sa, par0, cm);
        int nl = 0;
        for (int st = 0; st < nst; ++st) nl += enqueue_step<T>(Uc, Pc, Uo, sc, sa, nullptr, (par0 + st) & 1, nullptr, true, cm);
        return nl;
    }

    // Minv P of the receiver slots into rz[par] (symplectic runs, before the
    // first step of a run or of a recomputed segment).
    template <class T> void rz_init(const T *Pc, int par)
    {
        if (nk == 0) return;
        const int nrz = std::max(nk, 1);
        tet_rz_init_kernel<T><<<(nk + 127) / 128, 128, 0, stream>>>(nk, d_kslot.as<int>(), nnode, d_minv.as<T>(), Pc,
                                                                     d_rz.as<T>() + (size_t)par * nrz);
    }

    // Uploads the receivers, the dipole table and the per-substep source
    // values of an nsteps run from the current time; returns the source
    // arguments of the step kernels and fills the sample times.
    SrcArgs prepare_run(int nsteps, const Schedule &sc, std::vector<double> &times, double &t_end)
    {
        const int tf = P.time_frequency;
        nobs = (int)rec_edges.size();
        nsamp = nsteps > 0 ? (nsteps - 1) / tf + 1 : 0;
        ncols = 4;
        std::vector<int> re;
        std::vector<double> rw;
        for (int r = 0; r < nobs; ++r) {
            re.insert(re.end(), rec_edges[r].begin(), rec_edges[r].end());
            rw.insert(rw.end(), rec_w[r].begin(), rec_w[r].end());
        }
        // the receivers' distinct slots (sorted), each receiver slot's entry
        // among them, and the flag bit that makes the step kernel keep
        // Minv P of those slots
        std::vector<int> ks(re.begin(), re.end());
        std::sort(ks.begin(), ks.end());
        ks.erase(std::unique(ks.begin(), ks.end()), ks.end());
        std::vector<int> rk(re.size());
        for (size_t q = 0; q < re.size(); ++q) rk[q] = (int)(std::lower_bound(ks.begin(), ks.end(), re[q]) - ks.begin());
        nk = (int)ks.size();
        if (!kidx_valid || ks != rec_ks) {   // the receiver slots changed: flag bits and slot -> entry table
            for (int e : rec_ks) { pec_h[e] &= (unsigned char)~kRecBit; flags_dirty = true; }
            for (int e : ks) { pec_h[e] |= kRecBit; flags_dirty = true; }
            std::vector<int> kidx(nslot, -1);
            for (int k = 0; k < nk; ++k) kidx[ks[k]] = k;
            up(d_kidx, kidx);
            rec_ks = ks;
            kidx_valid = true;
        }
        if (re.empty()) { re.assign(6, 0); rw.assign(18, 0.0); rk.assign(6, 0); }
        if (ks.empty()) ks.push_back(0);
        up(d_rec_e, re);
        up(d_rec_w, rw);
        up(d_rec_k, rk);
        up(d_kslot, ks);
        d_rz.ensure(2 * ks.size() * (fp64 ? 8 : 4));
        d_rz.zero(stream);
        size_t ntr = (size_t)std::max(nobs, 1) * std::max(nsamp, 1) * 4;
        d_tr.ensure(ntr * 8);
        d_tr.zero(stream);
        // source entries sorted by slot, entries of one slot in dipole order
        std::vector<std::array<int, 2>> ent;   // (slot, dipole * 6 + l)
        for (size_t k = 0; k < dips.size(); ++k)
            for (int l = 0; l < 6; ++l) ent.push_back({dips[k].slot[l], (int)(6 * k + l)});
        std::stable_sort(ent.begin(), ent.end(), [](const std::array<int, 2> &x, const std::array<int, 2> &y) { return x[0] < y[0]; });
        std::vector<int> sslot, sdip;
        std::vector<double> scoef;
        for (auto &en : ent) {
            sslot.push_back(en[0]);
            sdip.push_back(en[1] / 6);
            scoef.push_back(dips[en[1] / 6].coef[en[1] % 6]);
        }
        int nsrc = (int)sslot.size();
        if (sslot.empty()) { sslot.push_back(0); sdip.push_back(0); scoef.push_back(0.0); }
        up(d_src_slot, sslot);
        up(d_src_coef, scoef);
        up(d_src_dip, sdip);
        if (flags_dirty) {
            EMS_CUDA(cudaMemcpyAsync(d_pec.p, pec_h.data(), nslot, cudaMemcpyHostToDevice, stream));
            flags_dirty = false;
        }
        size_t nd = std::max<size_t>(dips.size(), 1);
        std::vector<double> gv((size_t)std::max(nsteps, 1) * sc.nsub * nd, 0.0);
        times.assign(std::max(nsamp, 1), 0.0);
        double t = cur_time;
        for (int st = 0; st < nsteps; ++st) {
            for (int q = 0; q < sc.nsub; ++q)
                for (size_t k = 0; k < dips.size(); ++k) {
                    double tt = sc.symp ? t + sc.off[q] + 0.5 * sc.sub[q] : t;
                    gv[((size_t)st * sc.nsub + q) * nd + k] = tet_wave(dips[k].kind, dips[k].f0n, tt);
                }
            if (st % tf == 0) times[st / tf] = t;
            t += dtn;
        }
        t_end = t;
        up(d_src_g, gv);
        d_ctl.ensure(16);
        d_ctl.zero(stream);
        return SrcArgs{nsrc, d_src_slot.as<int>(), d_src_coef.as<double>(), d_src_dip.as<int>(), d_src_g.as<double>(),
                       d_ctl.as<int>(), (int)nd, sc.nsub, 0, 0};
    }

    // Snapshot s of the merged state of a recorded run: U and P in the run
    // precision, then (FP32) the compensation plane of P.
    size_t snap_bytes() const { return 2 * nslot * (fp64 ? 8 : 4) + (fp64 ? 0 : nslot * 2); }
    template <class T> void save_snapshot(int s, const T *U, const T *Pv)
    {
        char *b = d_snap.as<char>() + (size_t)s * snap_bytes();
        const size_t w = nslot * sizeof(T);
        EMS_CUDA(cudaMemcpyAsync(b, U, w, cudaMemcpyDeviceToDevice, stream));
        EMS_CUDA(cudaMemcpyAsync(b + w, Pv, w, cudaMemcpyDeviceToDevice, stream));
        if (!fp64) EMS_CUDA(cudaMemcpyAsync(b + 2 * w, d_comp.p, nslot * 2, cudaMemcpyDeviceToDevice, stream));
    }
    // Restores snapshot s into U, P and (FP32) P's compensation plane cp.
    template <class T> void load_snapshot(int s, T *U, T *Pv, __nv_bfloat16 *cp)
    {
        const char *b = d_snap.as<char>() + (size_t)s * snap_bytes();
        const size_t w = nslot * sizeof(T);
        EMS_CUDA(cudaMemcpyAsync(U, b, w, cudaMemcpyDeviceToDevice, stream));
        EMS_CUDA(cudaMemcpyAsync(Pv, b + w, w, cudaMemcpyDeviceToDevice, stream));
        if (cp) EMS_CUDA(cudaMemcpyAsync(cp, b + 2 * w, nslot * 2, cudaMemcpyDeviceToDevice, stream));
    }

    template <class T> void run_t(int nsteps)
    {
        if (!ready) setup();
        const Schedule sc = schedule();
        const bool symp = sc.symp;
        // record for ems_tetfem_backward: symplectic runs from the reset state
        const bool record = ckpt_nsnap > 0 && symp && fresh && nsteps > 0;
        rec_nsteps = -1;
        bar_used = false;   // set when this run enqueues a persistent launch
        std::vector<double> times;
        double t_end = 0.0;
        const SrcArgs sa = prepare_run(nsteps, sc, times, t_end);
        const unsigned nb128 = (unsigned)((nnode + 127) / 128);
        // symplectic: P in place, U alternating between Uc and Uo; leapfrog
        // ring: Uc = E^n, Pc = E^{n-1}, Uo = scratch for E^{n+1}
        T *Uc = d_U.as<T>(), *Pc = d_P.as<T>(), *Uo = d_Uold.as<T>();
        const Comp cm = symp ? comp() : Comp{};   // leapfrog runs are not compensated
        // CUDA graphs of kGraphSteps steps, replayed.  kGraphSteps is a
        // multiple of 3 and even, so the leapfrog ring, the symplectic U
        // pair and the counter parity return to the assignment a graph was
        // captured with; a single symp4 or symp2 step swaps the U pair and
        // the parity together, so a recorded run keeps one graph per
        // assignment.
        constexpr int kGraphSteps = 12;
        struct StepGraph {   // destroyed on every exit path
            cudaGraph_t g = nullptr;
            cudaGraphExec_t exec = nullptr;
            const void *start = nullptr;
            int par = 0;
            int launches = 0;   // kernel launches of one replay
            ~StepGraph()
            {
                if (exec) cudaGraphExecDestroy(exec);
                if (g) cudaGraphDestroy(g);
            }
        } graph[2], cand[kShapes];
        struct Events {   // timing of the launch-shape candidates
            cudaEvent_t e[kShapes * kTuneRounds + 1] = {};
            ~Events()
            {
                for (cudaEvent_t x : e)
                    if (x) cudaEventDestroy(x);
            }
        } tev;
        int par = 0;   // parity of the next step's counter copy
        auto capture = [&](StepGraph &G, T *u, T *p, T *o, int par0) {
            G.start = u;
            G.par = par0;
            int nl = 0;
            EMS_CUDA(cudaStreamSynchronize(stream));
            EMS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            try {
                nl += enqueue_steps<T>(kGraphSteps, u, p, o, sc, sa, par0, cm);
            } catch (...) {   // end the capture before the error leaves
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(stream, &g);
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                throw;
            }
            cudaError_t ce = cudaStreamEndCapture(stream, &G.g);
            if (ce != cudaSuccess) throw Error{EMS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce)};
            ce = cudaGraphInstantiate(&G.exec, G.g, 0);
            if (ce != cudaSuccess) throw Error{EMS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce)};
            G.launches = nl;
        };
        long long launches = 0;
        auto advance = [&](int k) {
            const StepGraph *sg = nullptr;
            for (auto &G : graph)
                if (G.exec && G.start == Uc && G.par == par) sg = &G;
            const int nrep = sg ? k / kGraphSteps : 0;
            for (int r = 0; r < nrep; ++r) EMS_CUDA(cudaGraphLaunch(sg->exec, stream));
            launches += (long long)nrep * (sg ? sg->launches : 0);
            const int rest = k - nrep * kGraphSteps;
            launches += enqueue_steps<T>(rest, Uc, Pc, Uo, sc, sa, par, cm);
            par ^= rest & 1;
        };
        int seg_len = 0, nseg = 0;
        if (record) {
            seg_len = (nsteps + ckpt_nsnap - 1) / ckpt_nsnap;
            nseg = (nsteps + seg_len - 1) / seg_len;
            d_snap.alloc((size_t)nseg * snap_bytes());
        }
        // launch-shape tuning in the first unrecorded run long enough: every
        // candidate's graph of kGraphSteps steps starts from the assignment
        // (Uc, parity 0) and returns to it, so they are captured up front
        int cl[kShapes], ncl = 0;   // the candidates this run can launch
        for (int ci = 0; ci < kShapes; ++ci)
            if (ci != kShapePersist || can_persist(symp)) cl[ncl++] = ci;
        const int tune_steps = ncl * kTuneRounds * kGraphSteps;
        const bool tuning = !step_tuned && !record && nsteps >= tune_steps + kGraphSteps;
        if (tuning) {
            int kept = 0;
            for (int i = 0; i < ncl; ++i) {
                set_shape(cl[i]);
                try {
                    capture(cand[cl[i]], Uc, Pc, Uo, 0);
                } catch (const Error &) {   // a device without cooperative launches in graphs: no persistent step
                    if (cl[i] != kShapePersist) throw;
                    persist_cap = 0;
                    continue;
                }
                cl[kept++] = cl[i];
            }
            ncl = kept;
            for (auto &x : tev.e) EMS_CUDA(cudaEventCreate(&x));
        } else if ((record ? seg_len : nsteps) >= kGraphSteps) {
            capture(graph[0], Uc, Pc, Uo, 0);
            if (record && symp && sc.nsub % 2 == 1) capture(graph[1], Uo, Pc, Uc, 1);
        }
        if (bar_used) EMS_CUDA(cudaMemsetAsync(d_bar.p, 0, 8, stream));   // the persistent step's barrier
        EMS_CUDA(cudaEventRecord(ev0, stream));
        if (symp) {
            tet_drift_kernel<T><<<nb128, 128, 0, stream>>>(nnode, d_minv.as<T>(), Pc, Uc, (T)sc.hfirst);
            rz_init<T>(Pc, 0);
            launches += nk > 0 ? 2 : 1;
        }
        int done = 0;   // steps advanced by the tuning graphs
        if (tuning) {
            for (int r = 0; r < kTuneRounds; ++r)
                for (int i = 0; i < ncl; ++i) {
                    EMS_CUDA(cudaEventRecord(tev.e[r * ncl + i], stream));
                    EMS_CUDA(cudaGraphLaunch(cand[cl[i]].exec, stream));
                    launches += cand[cl[i]].launches;
                }
            EMS_CUDA(cudaEventRecord(tev.e[ncl * kTuneRounds], stream));
            EMS_CUDA(cudaEventSynchronize(tev.e[ncl * kTuneRounds]));
            float best[kShapes] = {};
            for (int r = 0; r < kTuneRounds; ++r)
                for (int i = 0; i < ncl; ++i) {
                    float ms = 0.0f;
                    EMS_CUDA(cudaEventElapsedTime(&ms, tev.e[r * ncl + i], tev.e[r * ncl + i + 1]));
                    if (r == 0 || ms < best[i]) best[i] = ms;
                }
            int pi = 0;
            for (int i = 1; i < ncl; ++i)
                if (best[i] < best[pi]) pi = i;
            const int pick = cl[pi];
            if (std::getenv("EMS_TET_TUNE_LOG")) {   // diagnostic: the candidates' times per step
                static const char *names[kShapes] = {"node32", "node64", "node128", "node256", "slot", "persist"};
                std::fprintf(stderr, "tet step tuning (us per step):");
                for (int i = 0; i < ncl; ++i) std::fprintf(stderr, " %s %.3f", names[cl[i]], 1e3 * best[i] / kGraphSteps);
                std::fprintf(stderr, "\n");
            }
            set_shape(pick);
            step_tuned = true;
            std::swap(graph[0].g, cand[pick].g);
            std::swap(graph[0].exec, cand[pick].exec);
            graph[0].start = cand[pick].start;
            graph[0].par = cand[pick].par;
            graph[0].launches = cand[pick].launches;
            done = ncl * kTuneRounds * kGraphSteps;
        }
        if (record) {
            // snapshot of the merged state at the start of every segment
            for (int s = 0; s < nseg; ++s) {
                save_snapshot(s, Uc, Pc);
                advance(std::min(seg_len, nsteps - s * seg_len));
            }
        } else {
            advance(nsteps - done);
        }
        if (symp) {
            tet_drift_kernel<T><<<nb128, 128, 0, stream>>>(nnode, d_minv.as<T>(), Pc, Uc, (T)(-sc.hfirst));
            ++launches;
        }
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaEventRecord(ev1, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        {   // keep the current buffers: U (symplectic) or the ring U = E^n, P = E^{n-1}
            void *u = Uc, *p = Pc, *o = Uo;
            d_U.p = u; d_P.p = p; d_Uold.p = o;
        }
        float ms = 0;
        EMS_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        last_ms = ms;
        last_launches = launches;
        cur_time = t_end;
        fresh = nsteps == 0 && fresh;
        if (record) { rec_nsteps = nsteps; rec_seg = seg_len; rec_sa = sa; }
        const size_t ntr = (size_t)std::max(nobs, 1) * std::max(nsamp, 1) * 4;
        traces.assign(ntr, 0.0);
        EMS_CUDA(cudaMemcpy(traces.data(), d_tr.p, ntr * 8, cudaMemcpyDeviceToHost));
        traces.resize((size_t)nobs * nsamp * 4);
        for (int r = 0; r < nobs; ++r)
            for (int s = 0; s < nsamp; ++s) traces[((size_t)r * nsamp + s) * 4] = times[s] * tscale;
        if (bar_used) {   // a grid barrier of the persistent step that gave up
            int err = 0;
            EMS_CUDA(cudaMemcpy(&err, d_bar.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost));
            if (err)
                throw Error{EMS_ERR_DEVICE_TIMEOUT,
                            "a grid barrier of the persistent step timed out; the fields are invalid (reset the handle)"};
        }
    }

    // ---- discrete adjoint of the recorded run
    // Receiver terms grouped by edge slot and by node for
    // tet_receiver_gather_kernel and tet_receiver_drift_kernel.
    struct RecAdj {
        DevBuf sl_slot, sl_ptr, term_rc, term_w, nd_node, nd_map, a_scr;
        int nsl = 0, nnd = 0;
    };
    void build_receiver_adjoint(RecAdj &ra)
    {
        std::vector<int> sl_slot, sl_ptr{0}, term_rc, nd_node, nd_map;
        std::vector<double> term_w;
        std::vector<std::vector<std::pair<int, double>>> terms;
        std::unordered_map<int, int> slot_idx, node_idx;
        for (int r = 0; r < nobs; ++r)
            for (int l = 0; l < 6; ++l) {
                const int e = rec_edges[r][l];
                auto it = slot_idx.find(e);
                int k;
                if (it == slot_idx.end()) {
                    k = (int)sl_slot.size();
                    slot_idx[e] = k;
                    sl_slot.push_back(e);
                    terms.emplace_back();
                } else {
                    k = it->second;
                }
                for (int c = 0; c < 3; ++c) terms[k].push_back({3 * r + c, rec_w[r][3 * l + c]});
            }
        for (size_t k = 0; k < sl_slot.size(); ++k) {
            for (auto &tm : terms[k]) { term_rc.push_back(tm.first); term_w.push_back(tm.second); }
            sl_ptr.push_back((int)term_rc.size());
            const int v = sl_slot[k] / 7, d = sl_slot[k] % 7;
            auto it = node_idx.find(v);
            int i;
            if (it == node_idx.end()) {
                i = (int)nd_node.size();
                node_idx[v] = i;
                nd_node.push_back(v);
                nd_map.insert(nd_map.end(), 7, -1);
            } else {
                i = it->second;
            }
            nd_map[7 * i + d] = (int)k;
        }
        ra.nsl = (int)sl_slot.size();
        ra.nnd = (int)nd_node.size();
        if (sl_slot.empty()) { sl_slot.push_back(0); term_rc.push_back(0); term_w.push_back(0.0); nd_node.push_back(0); nd_map.assign(7, -1); }
        up(ra.sl_slot, sl_slot); up(ra.sl_ptr, sl_ptr); up(ra.term_rc, term_rc); up(ra.term_w, term_w);
        up(ra.nd_node, nd_node); up(ra.nd_map, nd_map);
        ra.a_scr.alloc(std::max(ra.nsl, 1) * sizeof(double));
    }

    // dJ/deps per tetrahedron (FP64) for dJ/dtraces tg (nobs x nsamp x 4,
    // column 0 ignored) of the recorded run.  Segments are recomputed from
    // their snapshots (keeping Minv P of every substep), then swept backward.
    template <class T> void backward_t(const double *tg, double *grad, double *grad_sigma)
    {
        const Schedule sc = schedule();
        const int N = rec_nsteps, L = rec_seg, nseg = (N + L - 1) / L, tf = P.time_frequency, nsub = sc.nsub;
        const unsigned nbt = (unsigned)((ntet + 255) / 256), nb128 = (unsigned)((nnode + 127) / 128);
        const unsigned nbv = (unsigned)((nnode + 127) / 128), nbv2 = nbv;
        // adjoint sources per sample: r[s][rec][c]
        std::vector<double> rs((size_t)std::max(nsamp, 1) * std::max(nobs, 1) * 3, 0.0);
        for (int r = 0; r < nobs; ++r)
            for (int s = 0; s < nsamp; ++s)
                for (int c = 0; c < 3; ++c) rs[((size_t)s * nobs + r) * 3 + c] = tg[((size_t)r * nsamp + s) * 4 + 1 + c];
        DevBuf d_rs, Wb, Pb, Pb2, Q, zbuf, ybuf, Uw, Uw2, Pw, contrib, d_grad, pstore, zr, cw, cb;
        up(d_rs, rs);
        RecAdj ra;
        build_receiver_adjoint(ra);
        const size_t w = sizeof(T);
        Wb.alloc(nslot * w); Wb.zero(stream);
        Pb.alloc(nslot * w); Pb.zero(stream);
        Pb2.alloc(nslot * w);
        Q.alloc(28 * nnode * 8); Q.zero(stream);
        zbuf.alloc(((size_t)L * nsub + 1) * nslot * w);
        ybuf.alloc((size_t)L * nsub * nslot * w);
        Uw.alloc(nslot * w); Uw2.alloc(nslot * w); Pw.alloc(nslot * w);
        // FP32: compensation planes of the recomputed forward state (restored
        // from each snapshot) and of the adjoint state (Pbar in the role of
        // U, Wbar in the role of P), the latter carried across segments
        Comp cfw, cadj;
        if (!fp64) {
            cw.alloc(nslot * 2);
            cb.alloc(nslot * 2);
            cb.zero(stream);
            cfw = Comp{cw.as<__nv_bfloat16>()};
            cadj = Comp{cb.as<__nv_bfloat16>()};
        }
        if (has_loss) {   // P around every lossy middle kick of a segment, and the loss sensitivities
            pstore.alloc((size_t)L * 2 * nslot * w);
            zr.alloc(nnode * 8);
            zr.zero(stream);
        }
        const SrcArgs sa = rec_sa;   // the recorded run's source tables are still on the device
        T *zb = zbuf.as<T>(), *yb = ybuf.as<T>();
        T *pb = Pb.as<T>(), *pb2 = Pb2.as<T>();   // Pbar alternates between the two
        for (int s = nseg - 1; s >= 0; --s) {
            const int n0 = s * L, n1 = std::min(N, n0 + L);
            load_snapshot<T>(s, Uw.as<T>(), Pw.as<T>(), cfw.p);
            EMS_CUDA(cudaMemcpyAsync(d_ctl.as<int>() + (n0 & 1), &n0, sizeof(int), cudaMemcpyHostToDevice, stream));
            // z[0] = Minv P at the start of step n0
            EMS_CUDA(cudaMemsetAsync(zb, 0, nslot * w, stream));
            tet_drift_kernel<T><<<nb128, 128, 0, stream>>>(nnode, d_minv.as<T>(), Pw.as<T>(), zb, T(1));
            T *uc = Uw.as<T>(), *pc = Pw.as<T>(), *uo = Uw2.as<T>();
            for (int n = n0; n < n1; ++n)
                enqueue_step<T>(uc, pc, uo, sc, sa, zb + ((size_t)(n - n0) * nsub + 1) * nslot, n & 1,
                                has_loss ? pstore.as<T>() + (size_t)(n - n0) * 2 * nslot : nullptr, false, cfw);
            for (int n = n1 - 1; n >= n0; --n) {
                for (int q = nsub - 1; q >= 0; --q) {
                    // the drift before kick (n, q): same step (q > 0), the
                    // previous step's last one, or the initial half drift
                    const double c = q > 0 ? sc.c[q - 1] : (n > 0 ? sc.c[nsub - 1] : sc.hfirst);
                    T *y = yb + ((size_t)(n - n0) * nsub + q) * nslot;
                    // Wbar -= a K Pbar; Pbar += c Minv Wbar (y = Minv Wbar kept)
                    if (has_loss && q == nsub / 2) {
                        // the lossy middle kick: Pbar = g Pbar before the
                        // adjoint kick, Pbar = g Pbar + c Minv Wbar after it
                        const T *pp = pstore.as<T>() + (size_t)(n - n0) * 2 * nslot;
                        tet_loss_adjoint_kernel<T><<<nbv2, 128, 0, stream>>>(nnode, d_damp.as<T>(), pb, pp + nslot, pp,
                                                                            zr.as<double>());
                        substep<T, 0, 2>(pb, pb2, Wb.as<T>(), nullptr, (T)sc.sub[q], (T)c, SrcArgs{}, y, nullptr, nullptr,
                                         RecArgs<T>{}, cadj);
                    } else {
                        substep<T, 0>(pb, pb2, Wb.as<T>(), nullptr, (T)sc.sub[q], (T)c, SrcArgs{}, y, nullptr, nullptr,
                                      RecArgs<T>{}, cadj);
                    }
                    std::swap(pb, pb2);
                }
                if (n % tf == 0 && n > 0 && nobs > 0 && ra.nsl > 0) {
                    const T *z = zb + (size_t)(n - n0) * nsub * nslot;
                    tet_receiver_gather_kernel<T><<<(ra.nsl + 255) / 256, 256, 0, stream>>>(
                        ra.nsl, ra.sl_slot.as<int>(), ra.sl_ptr.as<int>(), ra.term_rc.as<int>(), ra.term_w.as<double>(),
                        d_rs.as<double>() + (size_t)(n / tf) * nobs * 3, ra.a_scr.as<double>(), Wb.as<T>(), nnode);
                    if (sc.sub[nsub - 1] != 0.0 && ra.nnd > 0)
                        tet_receiver_drift_kernel<T><<<(ra.nnd + 127) / 128, 128, 0, stream>>>(
                            ra.nnd, ra.nd_node.as<int>(), ra.nd_map.as<int>(), ra.a_scr.as<double>(), pb, d_minv.as<T>(),
                            z, Q.as<double>(), 0.5 * sc.sub[nsub - 1], nnode);
                }
            }
            // the drifts of this segment: y at [k], z at [k] (k = nsub (n - n0) + q)
            tet_grad_accumulate_kernel<T><<<nb128, 128, 0, stream>>>(nnode, nslot, (n1 - n0) * nsub, nsub, n0, (T)sc.c[0],
                                                                   (T)sc.c[1], (T)sc.c[2], (T)sc.hfirst, yb, zb,
                                                                   Q.as<double>());
            EMS_CUDA(cudaGetLastError());
        }
        contrib.alloc(6 * ntet * 8);
        contrib.zero(stream);
        d_grad.alloc(ntet * 8);
        tet_grad_node_kernel<<<nbv, 128, 0, stream>>>(nnode, d_pec.as<unsigned char>(), d_inc_ptr.as<int>(), d_inc.as<int>(),
                                                      d_eps.as<double>(), Q.as<double>(), contrib.as<double>());
        tet_grad_gather_kernel<<<nbt, 256, 0, stream>>>(ntet, d_tet_edge.as<int>(), d_pec.as<unsigned char>(),
                                                        d_inc_ptr.as<int>(), d_inc.as<int>(), contrib.as<double>(),
                                                        d_grad.as<double>());
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaMemcpyAsync(grad, d_grad.p, ntet * 8, cudaMemcpyDeviceToHost, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        loss_gradient(zr, grad, grad_sigma);
    }

    // Loss-rate terms of the gradient (host, FP64): each loss factor g_v =
    // exp(-rho_v dt/2) gives dJ/drho_v = -(dt/2) g_v zr_v, and rho_v =
    // sum sigma_T c_Tv / den_v (c_Tv the loss weights of T at v) gives
    // dJ/dsigma_T = sum_v dJ/drho_v c_Tv / den_v and dJ/deps_T -= sum_v
    // dJ/drho_v rho_v c_Tv / den_v.  grad_sigma is per S/m.
    void loss_gradient(const DevBuf &zr, double *grad, double *grad_sigma)
    {
        if (grad_sigma)
            for (size_t t = 0; t < ntet; ++t) grad_sigma[t] = 0.0;
        if (!has_loss) return;
        std::vector<double> z(nnode);
        EMS_CUDA(cudaMemcpy(z.data(), zr.p, nnode * 8, cudaMemcpyDeviceToHost));
        double wsq[6][6];
        for (int p = 0; p < 6; ++p) {
            const Shape sh = make_shape(p);
            for (int l = 0; l < 6; ++l) wsq[p][l] = sh.wsq[l];
        }
        const double sig_unit = tscale / kEps0;   // d sigma_normalised / d sigma
        for (size_t v = 0; v < nnode; ++v) {
            if (lden_h[v] <= 0.0) continue;
            const double gr = -0.5 * dtn * std::exp(-0.5 * dtn * rho_h[v]) * z[v];
            for (int d = 0; d < 7; ++d) {
                const size_t e = 7 * v + d;
                if (pec_h[e] & kPecBit) continue;
                for (int q = inc_ptr_h[e]; q < inc_ptr_h[e + 1]; ++q) {
                    const int t = inc_h[q] >> 3, l = inc_h[q] & 7, p = t % 6;
                    const double wv = wsq[p][l] / lden_h[v];
                    if (grad_sigma) grad_sigma[t] += gr * wv * sig_unit;
                    grad[t] -= gr * rho_h[v] * wv;
                }
            }
        }
    }

    // Discrete energy H = 1/2 P.Minv P + 1/2 U.K U of the current
    // symplectic state, per shot, in FP64 on the GPU.
    void energy(double *out, int n)
    {
        if (!schedule().symp) throw Error{EMS_ERR_UNSUPPORTED, "the discrete energy is defined for the symplectic integrators"};
        EMS_CHECK_ARG(out && n == (int)shots.size(), "energy needs one value per shot");
        if (!ready) setup();
        DevBuf u64, f64, e, part, res;
        f64.alloc(nslot * 8);
        e.alloc(nnode * 8);
        part.alloc(512 * 8);
        res.alloc(shots.size() * 8);
        const DevBuf *u = &d_U;
        if (!fp64) {
            u64.alloc(nslot * 8);
            widen_kernel<float><<<(unsigned)((nslot + 255) / 256), 256, 0, stream>>>(nslot, d_U.as<float>(), u64.as<double>());
            u = &u64;
        }
        applyK64(*u, f64);
        const unsigned nb = (unsigned)((nnode + 127) / 128);
        if (fp64)
            tet_energy_node_kernel<double><<<nb, 128, 0, stream>>>(nnode, d_minv.as<double>(), d_P.as<double>(),
                                                                    d_U.as<double>(), f64.as<double>(), e.as<double>());
        else
            tet_energy_node_kernel<float><<<nb, 128, 0, stream>>>(nnode, d_minv.as<float>(), d_P.as<float>(), d_U.as<float>(),
                                                                   f64.as<double>(), e.as<double>());
        for (size_t k = 0; k < shots.size(); ++k) {
            const Shot &S = shots[k];
            const size_t nv = (size_t)(S.nx + 1) * (S.ny + 1) * (S.nz + 1);
            dot_partial_kernel<<<512, 256, 0, stream>>>(nv, e.as<double>() + S.node0, nullptr, part.as<double>());
            dot_finish_kernel<<<1, 512, 0, stream>>>(512, part.as<double>(), res.as<double>() + k);
        }
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaMemcpyAsync(out, res.p, shots.size() * 8, cudaMemcpyDeviceToHost, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    void backward(const double *tg, size_t ntg, double *grad, size_t ngrad, double *grad_sigma)
    {
        if (rec_nsteps < 0)
            throw Error{EMS_ERR_STATE, "no recorded run: call ems_tetfem_set_checkpoints, ems_reset, then ems_run"};
        EMS_CHECK_ARG(tg && grad, "trace gradient and output required");
        EMS_CHECK_ARG(ntg == (size_t)nobs * nsamp * 4, "trace gradient must have nrec * nsamp * 4 values");
        EMS_CHECK_ARG(ngrad == ntet, "gradient must have one value per tetrahedron");
        if (fp64) backward_t<double>(tg, grad, grad_sigma); else backward_t<float>(tg, grad, grad_sigma);
    }

    void run(int nsteps) override
    {
        EMS_CHECK_ARG(nsteps >= 0, "num_steps must be >= 0");
        if (fp64) run_t<double>(nsteps); else run_t<float>(nsteps);
        check_finite({{d_U.p, nslot}, {d_P.p, nslot}}, fp64);
    }

    size_t field_size(int which) const override
    {
        if (which < 0 || which > 1) throw Error{EMS_ERR_INVALID_ARGUMENT, "field index must be 0 (U) or 1 (P)"};
        return nslot;
    }
    // Fields cross the API in slot order (e = 7 node + d) and live on the
    // device in the plane layout (fslot).  With a compensation plane lo
    // (FP32 symplectic handles) the value is hi + lo, split again on upload.
    template <class T> void download_slots(const DevBuf &b, double *out, const __nv_bfloat16 *lo = nullptr) const
    {
        std::vector<T> tmp(nslot);
        EMS_CUDA(cudaMemcpy(tmp.data(), b.p, nslot * sizeof(T), cudaMemcpyDeviceToHost));
        std::vector<uint16_t> lw(lo ? nslot : 0);
        if (lo) EMS_CUDA(cudaMemcpy(lw.data(), lo, nslot * 2, cudaMemcpyDeviceToHost));
        for (size_t e = 0; e < nslot; ++e) {
            const size_t f = fslot(e, nnode);
            out[e] = (double)tmp[f] + (lo ? (double)bf16_to_float(lw[f]) : 0.0);
        }
    }
    template <class T> void upload_slots(DevBuf &b, const double *in, __nv_bfloat16 *lo = nullptr) const
    {
        std::vector<T> tmp(nslot);
        std::vector<uint16_t> lw(lo ? nslot : 0);
        for (size_t e = 0; e < nslot; ++e) {
            const size_t f = fslot(e, nnode);
            tmp[f] = (T)in[e];
            if (lo) lw[f] = float_to_bf16((float)(in[e] - (double)tmp[f]));
        }
        EMS_CUDA(cudaMemcpy(b.p, tmp.data(), nslot * sizeof(T), cudaMemcpyHostToDevice));
        if (lo) EMS_CUDA(cudaMemcpy(lo, lw.data(), nslot * 2, cudaMemcpyHostToDevice));
    }
    // bfloat16 <-> float on the host: the upper half of the binary32
    // pattern, rounded to nearest even on the way down (NaN kept quiet).
    static float bf16_to_float(uint16_t h)
    {
        const uint32_t u = (uint32_t)h << 16;
        float f;
        std::memcpy(&f, &u, 4);
        return f;
    }
    static uint16_t float_to_bf16(float f)
    {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
        u += 0x7fffu + ((u >> 16) & 1u);
        return (uint16_t)(u >> 16);
    }
    // The compensation plane of P (which == 1) of an FP32 symplectic
    // handle, else nullptr.
    __nv_bfloat16 *comp_plane(int which) const
    {
        const Comp c = comp();
        if (!c.p || !schedule().symp || which != 1) return nullptr;
        return c.p;
    }
    void get_field(int which, double *out) const override
    {
        const DevBuf &b = which == 0 ? d_U : d_P;
        if (fp64) download_slots<double>(b, out); else download_slots<float>(b, out, comp_plane(which));
    }
    void set_field(int which, const double *in) override
    {
        DevBuf &b = which == 0 ? d_U : d_P;
        fresh = false;
        if (fp64) upload_slots<double>(b, in); else upload_slots<float>(b, in, comp_plane(which));
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

    // f = K u through the force-only fused step (P = f = 0, a = -1 leaves
    // P = K u), in slot order on both sides.
    void apply_stiffness(const double *u, double *f)
    {
        size_t w = fp64 ? 8 : 4;
        DevBuf in, out;
        in.alloc(nslot * w);
        out.alloc(nslot * w);
        out.zero(stream);
        const unsigned nbv = (unsigned)((nnode + step_block - 1) / step_block);
        auto body = [&](auto tag) {
            using T = decltype(tag);
            EMS_CUDA(cudaStreamSynchronize(stream));
            upload_slots<T>(in, u);
            tet_step_kernel<T, 0, 0><<<nbv, step_block, 0, stream>>>(nnode, d_nrec.as<int2>(), d_pec.as<unsigned char>(), nullptr,
                                                              out.as<T>(), in.as<T>(), nullptr, nullptr, T(-1), T(0), SrcArgs{},
                                                              nullptr, nullptr, nullptr, nullptr, RecArgs<T>{}, Comp{});
            EMS_CUDA(cudaGetLastError());
            EMS_CUDA(cudaStreamSynchronize(stream));
            download_slots<T>(out, f);
        };
        if (fp64) body(double()); else body(float());
    }

    void reset() override
    {
        d_U.zero(stream); d_P.zero(stream); d_Uold.zero(stream);
        if (d_comp.p) d_comp.zero(stream);
        cur_time = 0.0;
        fresh = true;
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    void launch_shape(int b[3]) override
    {
        if (!ready) setup();
        if (slot_split) { b[0] = kSlotNodes; b[1] = 7; b[2] = 1; }
        else { b[0] = step_block; b[1] = b[2] = 1; }
    }

    void time_dominant(int launches, double *ms, double *bytes, std::string *name) override
    {
        if (!ready) setup();
        const unsigned nbv = (unsigned)((nnode + step_block - 1) / step_block);
        // the fused step of a substep in the handle's launch shape, as the time
        // loop runs it: a CUDA graph of 12 launches (a = c = 0 leaves P
        // unchanged and copies U between the two buffers the loop
        // alternates), replayed; launched one by one, the kernels would wait
        // on the host's launch rate
        // (the persistent step: one idle launch of 12 steps, timed per substep)
        constexpr int kLaunches = 12;
        const Schedule sc = schedule();
        const bool pers = persist && can_persist(sc.symp);
        const int per_graph = pers ? kLaunches * sc.nsub : kLaunches;   // substeps of one replay
        cudaGraph_t g = nullptr;
        cudaGraphExec_t exec = nullptr;
        if (pers) EMS_CUDA(cudaMemsetAsync(d_bar.p, 0, 8, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        EMS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        try {
            if (pers) {
                auto body = [&](auto tag) {
                    using T = decltype(tag);
                    T *u = d_U.as<T>(), *p = d_P.as<T>(), *o = d_Uold.as<T>();
                    persist_launch<T>(kLaunches, u, p, o, sc, SrcArgs{}, 0, comp(), true);
                };
                if (fp64) body(double()); else body(float());
            } else {
                for (int r = 0; r < kLaunches; ++r) idle_step(nbv, r % 2);
            }
        } catch (...) {
            cudaGraph_t gg = nullptr;
            cudaStreamEndCapture(stream, &gg);
            if (gg) cudaGraphDestroy(gg);
            cudaGetLastError();
            throw;
        }
        cudaError_t ce = cudaStreamEndCapture(stream, &g);
        if (ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, g, 0);
        const int reps = std::max(1, launches / per_graph);
        if (ce == cudaSuccess) ce = cudaGraphLaunch(exec, stream);
        if (ce == cudaSuccess) ce = cudaEventRecord(ev0, stream);
        for (int r = 0; r < reps && ce == cudaSuccess; ++r) ce = cudaGraphLaunch(exec, stream);
        if (ce == cudaSuccess) ce = cudaEventRecord(ev1, stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream);
        float t = 0;
        if (ce == cudaSuccess) ce = cudaEventElapsedTime(&t, ev0, ev1);
        if (exec) cudaGraphExecDestroy(exec);
        if (g) cudaGraphDestroy(g);
        if (ce != cudaSuccess) throw Error{EMS_ERR_CUDA, std::string("dominant-kernel timing: ") + cudaGetErrorString(ce)};
        if (pers) {
            int err = 0;
            EMS_CUDA(cudaMemcpy(&err, d_bar.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost));
            if (err) throw Error{EMS_ERR_DEVICE_TIMEOUT, "a grid barrier of the persistent step timed out"};
        }
        *ms = t / (reps * per_graph);
        const size_t w = fp64 ? 8 : 4;
        // unique bytes of one substep: node records (8 B per node) + U read
        // once (the neighbours' reads hit L1/L2) + P read and written + U
        // written + packed mass blocks + slot flags (+ FP32: P's bfloat16
        // compensation plane read and written)
        *bytes = (double)nnode * 8 + (double)nslot * 4 * w + (double)(28 * nnode) * w + (double)nslot +
                 (fp64 ? 0.0 : (double)nslot * 2 * 2);
        if (pers) *name = fp64 ? "tet_persist_kernel<double> (per substep)" : "tet_persist_kernel<float> (per substep)";
        else if (slot_split) *name = fp64 ? "tet_slot_kernel<double>" : "tet_slot_kernel<float>";
        else *name = fp64 ? "tet_step_kernel<double>" : "tet_step_kernel<float>";
    }
};

double tet_wave_value(int kind, double f0, double t) { return tet_wave(kind, f0, t); }
double tet_stability_constant(int integrator) { return stability_constant(integrator); }

Sim *make_tetfem(const ems_tetfem_params *p)
{
    EMS_CHECK_ARG(p != nullptr, "parameters required");
    EMS_CHECK_ARG(p->order == 1 || p->order == 2, "Nedelec order must be 1 or 2");
    std::vector<std::array<int, 3>> c{{p->cells[0], p->cells[1], p->cells[2]}};
    if (p->order == 2) return make_tet2(p, c);
    return new TetFemSim(p, c);
}

Sim *make_tetbatch(const ems_tetfem_params *p, int nshots, const int *cells)
{
    EMS_CHECK_ARG(p != nullptr, "parameters required");
    EMS_CHECK_ARG(nshots >= 1 && cells != nullptr, "need at least one shot");
    EMS_CHECK_ARG(p->order == 1 || p->order == 2, "Nedelec order must be 1 or 2");
    std::vector<std::array<int, 3>> c(nshots);
    for (int s = 0; s < nshots; ++s) c[s] = {cells[3 * s], cells[3 * s + 1], cells[3 * s + 2]};
    if (p->order == 2) return make_tet2(p, c);
    return new TetFemSim(p, c);
}

void tetfem_set_material(Sim *s, const double *eps_r, const double *sigma)
{
    if (is_tet2(s)) return tet2_set_material(s, eps_r, sigma);
    static_cast<TetFemSim *>(s)->set_material(eps_r, sigma);
}

void tetfem_add_dipole(Sim *s, const double pos[3], const double dir[3], int waveform, double f0, double amp)
{
    tetbatch_add_dipole(s, 0, pos, dir, waveform, f0, amp);
}

void tetbatch_add_dipole(Sim *s, int shot, const double pos[3], const double dir[3], int waveform, double f0, double amp)
{
    if (is_tet2(s)) return tet2_add_dipole(s, shot, pos, dir, waveform, f0, amp);
    auto *f = static_cast<TetFemSim *>(s);
    EMS_CHECK_ARG(shot >= 0 && shot < (int)f->shots.size(), "shot index out of range");
    const Shot &S = f->shots[shot];
    EMS_CHECK_ARG(pos && dir, "position and direction required");
    EMS_CHECK_ARG(waveform == EMS_WAVE_REFERENCE || waveform == EMS_WAVE_RICKER, "unknown waveform");
    EMS_CHECK_ARG(f0 > 0 && std::isfinite(amp), "f0 must be positive");
    double xn[3] = {pos[0] / f->P.h, pos[1] / f->P.h, pos[2] / f->P.h};
    const int lim[3] = {S.nx, S.ny, S.nz};
    for (int q = 0; q < 3; ++q) EMS_CHECK_ARG(xn[q] >= 0 && xn[q] <= lim[q], "dipole outside the domain");
    EMS_CHECK_ARG(f->dips.size() < 4096, "at most 4096 dipoles");
    double w[6][3];
    Dipole d{};
    f->locate(S, xn, w, d.slot);
    // loads on PEC slots vanish (the force is zero there)
    for (int l = 0; l < 6; ++l)
        d.coef[l] = (f->pec_h[d.slot[l]] & kPecBit) ? 0.0 : (w[l][0] * dir[0] + w[l][1] * dir[1] + w[l][2] * dir[2]) * amp;
    d.kind = waveform;
    d.f0n = f0 * f->tscale;
    f->dips.push_back(d);
    f->rec_nsteps = -1;
    for (int l = 0; l < 6; ++l)
        if (d.coef[l] != 0.0) f->pec_h[d.slot[l]] |= kSrcBit;
    f->flags_dirty = true;
}

void tetfem_add_receiver(Sim *s, const double pos[3]) { tetbatch_add_receiver(s, 0, pos); }

void tetbatch_add_receiver(Sim *s, int shot, const double pos[3])
{
    if (is_tet2(s)) return tet2_add_receiver(s, shot, pos);
    auto *f = static_cast<TetFemSim *>(s);
    EMS_CHECK_ARG(pos != nullptr, "position required");
    EMS_CHECK_ARG(shot >= 0 && shot < (int)f->shots.size(), "shot index out of range");
    const Shot &S = f->shots[shot];
    double xn[3] = {pos[0] / f->P.h, pos[1] / f->P.h, pos[2] / f->P.h};
    const int lim[3] = {S.nx, S.ny, S.nz};
    for (int q = 0; q < 3; ++q) EMS_CHECK_ARG(xn[q] >= 0 && xn[q] <= lim[q], "receiver outside the domain");
    double w[6][3];
    std::array<int, 6> e;
    f->locate(S, xn, w, e.data());
    std::array<double, 18> ww;
    for (int l = 0; l < 6; ++l)
        for (int q = 0; q < 3; ++q) ww[3 * l + q] = w[l][q];
    f->rec_edges.push_back(e);
    f->rec_w.push_back(ww);
    f->rec_nsteps = -1;
}

void tetfem_apply_stiffness(Sim *s, const double *u, double *f, size_t n)
{
    if (is_tet2(s)) return tet2_apply_stiffness(s, u, f, n);
    auto *t = static_cast<TetFemSim *>(s);
    EMS_CHECK_ARG(u && f, "input and output required");
    EMS_CHECK_ARG(n == t->nslot, "vector length must be 7*(nx+1)*(ny+1)*(nz+1)");
    t->apply_stiffness(u, f);
}

void tetfem_set_checkpoints(Sim *s, int nsnap)
{
    if (is_tet2(s)) return tet2_set_checkpoints(s, nsnap);
    static_cast<TetFemSim *>(s)->set_checkpoints(nsnap);
}
void tetfem_energy(Sim *s, double *out, int n)
{
    if (is_tet2(s)) return tet2_energy(s, out, n);
    static_cast<TetFemSim *>(s)->energy(out, n);
}

void tetfem_backward(Sim *s, const double *trace_grad, size_t ntg, double *grad_eps, double *grad_sigma, size_t ngrad)
{
    if (is_tet2(s)) return tet2_backward(s, trace_grad, ntg, grad_eps, grad_sigma, ngrad);
    static_cast<TetFemSim *>(s)->backward(trace_grad, ntg, grad_eps, ngrad, grad_sigma);
}

void tetfem_gradient(Sim *s, int nsteps, int nsnap, int kind, const double *obs, const double *band, double *misfit,
                     double *grad, double *grad_sigma, size_t ngrad)
{
    EMS_CHECK_ARG(nsteps > 0 && nsnap > 0, "nsteps and nsnap must be positive");
    EMS_CHECK_ARG(obs && misfit && grad, "observed traces, misfit and gradient required");
    EMS_CHECK_ARG(ngrad == (is_tet2(s) ? tet2_ntet(s) : static_cast<TetFemSim *>(s)->ntet),
                  "gradient must have one value per tetrahedron");
    tetfem_set_checkpoints(s, nsnap);
    s->reset();
    s->run(nsteps);
    std::vector<double> tg(s->traces.size());
    trace_misfit(kind, s->nobs, s->nsamp, s->traces.data(), obs, misfit, tg.data(), band);
    tetfem_backward(s, tg.data(), tg.size(), grad, grad_sigma, ngrad);
}

void tetfem_time_step(const Sim *s, double *dt, double *lim)
{
    if (is_tet2(s)) return tet2_time_step(s, dt, lim);
    auto *f = const_cast<TetFemSim *>(static_cast<const TetFemSim *>(s));
    if (!f->ready) f->setup();
    if (dt) *dt = f->dtn * f->tscale;
    if (lim) *lim = f->dt_lim_n * f->tscale;
}

}  // namespace ems
