// Yee FDTD on one GPU: the reference time loop of fdtd/fdtd_simulation.cpp
// (H from curl E 119-169, E from curl H 170-220, sources 222-239, receivers
// 261-303) on the reference's padded field layout (55-88), extended with
// per-cell materials and a convolutional PML.
//
// Arithmetic is written with explicitly rounded operations (no contraction
// into fused multiply-adds) in the reference's operand order, so the FP64
// path reproduces the reference bit for bit; the FP32 path runs the same
// operations in single precision.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <iomanip>

#include "ems_internal.hpp"

namespace ems {

__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }

// CPML coefficient profile along one axis, sampled at the derivative positions.
template <class T> struct Prof {
    const T *b, *a, *kinv;
    const unsigned char *on;
};

// Row (y) and plane (z) strides of the padded arrays and of the material
// grid, in elements (all arrays hold fewer than 2^32 elements).
struct FdtdStrides {
    unsigned ex_y, ex_z, ey_y, ey_z, ez_y, ez_z, hx_y, hx_z, hy_y, hy_z, hz_y, hz_z, m_y, m_z;
};

// (ca, cb) of one material, loaded as one vector.
template <class T> struct alignas(2 * sizeof(T)) CaCb {
    T ca, cb;
};

template <class T> struct FdtdArgs {
    T *Ex, *Ey, *Ez, *Hx, *Hy, *Hz;
    int nx, ny, nz;
    FdtdStrides st;
    T ch, ce;                      // uniform update coefficients dt/mu/h, dt/eps/h
    const uint16_t *mat;           // per-cell material id (MAT)
    const CaCb<T> *cab;            // per-material E coefficients (MAT)
    Prof<T> pe[3], ph[3];          // CPML profiles for E- and H-type derivatives (PML)
    T *psiE[3][2], *psiH[3][2];    // CPML auxiliary fields, full field size (PML)
    int in_lo[3], in_hi[3];        // per axis, the indices [lo, hi) where no profile is on (PML)
};

// Cells per thread along z (planes kFdtdKZ * blockIdx.z ...).  One: two
// cells per thread raised the E kernel's registers from 32 to 58 and its
// time at 512^3 from 1.76 to 2.93 ms.
constexpr int kFdtdKZ = 1;

// True when no thread of this block touches a CPML slab (the same for every
// thread of the block, so the slab tests and their flag loads are skipped
// uniformly; blocks that touch a slab test per thread as before).
template <class T> __device__ __forceinline__ bool block_outside_slabs(const FdtdArgs<T> &a)
{
    const int i0 = blockIdx.x * blockDim.x, j0 = blockIdx.y * blockDim.y, k0 = blockIdx.z * kFdtdKZ;
    return i0 >= a.in_lo[0] && i0 + (int)blockDim.x <= a.in_hi[0] && j0 >= a.in_lo[1] &&
           j0 + (int)blockDim.y <= a.in_hi[1] && k0 >= a.in_lo[2] && k0 + kFdtdKZ <= a.in_hi[2];
}

#define IEX(i, j, k) ((size_t)(i) + (size_t)(j) * (a.nx + 1) + (size_t)(k) * (a.nx + 1) * (a.ny + 2))
#define IEY(i, j, k) ((size_t)(i) + (size_t)(j) * (a.nx + 2) + (size_t)(k) * (a.nx + 2) * (a.ny + 1))
#define IEZ(i, j, k) ((size_t)(i) + (size_t)(j) * (a.nx + 2) + (size_t)(k) * (a.nx + 2) * (a.ny + 2))
#define IHX(i, j, k) ((size_t)(i) + (size_t)(j) * a.nx + (size_t)(k) * a.nx * (a.ny + 1))
#define IHY(i, j, k) ((size_t)(i) + (size_t)(j) * (a.nx + 1) + (size_t)(k) * (a.nx + 1) * a.ny)
#define IHZ(i, j, k) ((size_t)(i) + (size_t)(j) * (a.nx + 1) + (size_t)(k) * (a.nx + 1) * (a.ny + 1))

// d = ((p - q) - r) + s, the reference's evaluation order of a curl difference.
template <class T> __device__ __forceinline__ T curl4(T p, T q, T r, T s) { return radd(rsub(rsub(p, q), r), s); }

// One CPML-stretched update value: kinv1*d1 - kinv2*d2 + psi1 - psi2 with the
// auxiliary recursions psi = b psi + a d (oracle/orc_fdtd.c order).
template <class T>
__device__ __forceinline__ T pml_curl(T d1, T d2, const Prof<T> &p1, int s1, const Prof<T> &p2, int s2, T *psi1, T *psi2)
{
    T q1 = radd(rmul(p1.b[s1], *psi1), rmul(p1.a[s1], d1));
    T q2 = radd(rmul(p2.b[s2], *psi2), rmul(p2.a[s2], d2));
    *psi1 = q1;
    *psi2 = q2;
    return rsub(radd(rsub(rmul(p1.kinv[s1], d1), rmul(p2.kinv[s2], d2)), q1), q2);
}

// H from curl E at cell (i,j,k): fdtd_simulation.cpp:119-169.  Offsets are
// 32-bit, formed once per array and moved by the strides; E values shared
// by two components are loaded once.  Every load of the cell is issued
// before its first store (the three read-modify-writes touch distinct
// arrays and no other thread writes them), so a thread waits for one round
// of memory latency instead of one per component.
template <class T, bool PML>
__device__ __forceinline__ void fdtd_h_cell(const FdtdArgs<T> &a, int i, int j, int k, bool slab)
{
    const FdtdStrides &st = a.st;
    const unsigned oEx = i + j * st.ex_y + k * st.ex_z, oEy = i + j * st.ey_y + k * st.ey_z;
    const unsigned oEz = i + j * st.ez_y + k * st.ez_z;
    const unsigned px = i + j * st.hx_y + k * st.hx_z, py = i + j * st.hy_y + k * st.hy_z;
    const unsigned pz = i + j * st.hz_y + k * st.hz_z;
    const bool hx = i < a.nx, hy = j < a.ny, hz = k < a.nz;
    T ez11 = 0, ey1k = 0, ex1k = 0;   // Ez(i+1,j+1,k), Ey(i+1,j,k+1), Ex(i,j+1,k+1)
    T ez1 = 0, ey1 = 0, ex1 = 0, ez0 = 0, ey0 = 0, ex0 = 0, hx0 = 0, hy0 = 0, hz0 = 0;
    if (hx || hy) ez11 = __ldg(a.Ez + oEz + 1 + st.ez_y);
    if (hx || hz) ey1k = __ldg(a.Ey + oEy + 1 + st.ey_z);
    if (hy || hz) ex1k = __ldg(a.Ex + oEx + st.ex_y + st.ex_z);
    if (hx) {
        hx0 = a.Hx[px];
        ez1 = __ldg(a.Ez + oEz + 1);
        ey1 = __ldg(a.Ey + oEy + 1);
    }
    if (hy) {
        hy0 = a.Hy[py];
        ex1 = __ldg(a.Ex + oEx + st.ex_y);
        ez0 = __ldg(a.Ez + oEz + st.ez_y);
    }
    if (hz) {
        hz0 = a.Hz[pz];
        ey0 = __ldg(a.Ey + oEy + st.ey_z);
        ex0 = __ldg(a.Ex + oEx + st.ex_z);
    }
    if (hx) {
        if (slab && (a.ph[1].on[j] | a.ph[2].on[k])) {
            T c = pml_curl(rsub(ez11, ez1), rsub(ey1k, ey1), a.ph[1], j, a.ph[2], k, &a.psiH[0][0][px], &a.psiH[0][1][px]);
            a.Hx[px] = rsub(hx0, rmul(a.ch, c));
        } else {
            a.Hx[px] = rsub(hx0, rmul(a.ch, curl4(ez11, ez1, ey1k, ey1)));
        }
    }
    if (hy) {
        if (slab && (a.ph[2].on[k] | a.ph[0].on[i])) {
            T c = pml_curl(rsub(ex1k, ex1), rsub(ez11, ez0), a.ph[2], k, a.ph[0], i, &a.psiH[1][0][py], &a.psiH[1][1][py]);
            a.Hy[py] = rsub(hy0, rmul(a.ch, c));
        } else {
            a.Hy[py] = rsub(hy0, rmul(a.ch, curl4(ex1k, ex1, ez11, ez0)));
        }
    }
    if (hz) {
        if (slab && (a.ph[0].on[i] | a.ph[1].on[j])) {
            T c = pml_curl(rsub(ey1k, ey0), rsub(ex1k, ex0), a.ph[0], i, a.ph[1], j, &a.psiH[2][0][pz], &a.psiH[2][1][pz]);
            a.Hz[pz] = rsub(hz0, rmul(a.ch, c));
        } else {
            a.Hz[pz] = rsub(hz0, rmul(a.ch, curl4(ey1k, ey0, ex1k, ex0)));
        }
    }
}

template <class T, bool PML>
__global__ void __launch_bounds__(256) fdtd_h_kernel(FdtdArgs<T> a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i > a.nx || j > a.ny) return;
    const bool slab = PML && !block_outside_slabs(a);
#pragma unroll
    for (int kk = 0; kk < kFdtdKZ; ++kk) {
        const int k = blockIdx.z * kFdtdKZ + kk;
        if (k <= a.nz) fdtd_h_cell<T, PML>(a, i, j, k, slab);
    }
}

// (ca, cb) of one material through the read-only path.
__device__ __forceinline__ CaCb<float> load_cab(const CaCb<float> *p)
{
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    return {v.x, v.y};
}
__device__ __forceinline__ CaCb<double> load_cab(const CaCb<double> *p)
{
    const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    return {v.x, v.y};
}

// E from curl H at (i,j,k): fdtd_simulation.cpp:170-220, E = ca E + cb curl
// (ca, cb of the cell's material; uniform: E += ce curl).  As in the H
// update, all loads of the cell (fields, material ids, then their (ca, cb))
// are issued before the first store.
template <class T, bool MAT, bool PML>
__device__ __forceinline__ void fdtd_e_cell(const FdtdArgs<T> &a, int i, int j, int k, bool slab)
{
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const FdtdStrides &st = a.st;
    const unsigned oHx = i + j * st.hx_y + k * st.hx_z, oHy = i + j * st.hy_y + k * st.hy_z;
    const unsigned oHz = i + j * st.hz_y + k * st.hz_z;
    const unsigned px = i + j * st.ex_y + k * st.ex_z, py = i + j * st.ey_y + k * st.ey_z;
    const unsigned pz = i + j * st.ez_y + k * st.ez_z;
    const bool ex = j >= 1 && k >= 1, ey = i >= 1 && k >= 1, ez = i >= 1 && j >= 1;
    T hz_k = 0, hy_j = 0, hx_i = 0;   // Hz(i,j,k-1), Hy(i,j-1,k), Hx(i-1,j,k)
    T hz_jk = 0, hy_jk = 0, hx_ik = 0, hz_ik = 0, hy_ij = 0, hx_ij = 0, ex0 = 0, ey0 = 0, ez0 = 0;
    unsigned m0 = 0, m1 = 0, m2 = 0;
    if (ex || ey) hz_k = __ldg(a.Hz + oHz - st.hz_z);
    if (ex || ez) hy_j = __ldg(a.Hy + oHy - st.hy_y);
    if (ey || ez) hx_i = __ldg(a.Hx + oHx - 1);
    if (ex) {  // Ex, i in [0,nx]
        ex0 = a.Ex[px];
        hz_jk = __ldg(a.Hz + oHz - st.hz_y - st.hz_z);
        hy_jk = __ldg(a.Hy + oHy - st.hy_y - st.hy_z);
        if (MAT) m0 = __ldg(a.mat + (unsigned)(i < nx ? i : nx - 1) + (unsigned)(j - 1) * st.m_y + (unsigned)(k - 1) * st.m_z);
    }
    if (ey) {  // Ey, j in [0,ny]
        ey0 = a.Ey[py];
        hx_ik = __ldg(a.Hx + oHx - 1 - st.hx_z);
        hz_ik = __ldg(a.Hz + oHz - 1 - st.hz_z);
        if (MAT) m1 = __ldg(a.mat + (unsigned)(i - 1) + (unsigned)(j < ny ? j : ny - 1) * st.m_y + (unsigned)(k - 1) * st.m_z);
    }
    if (ez) {  // Ez, k in [0,nz]
        ez0 = a.Ez[pz];
        hy_ij = __ldg(a.Hy + oHy - 1 - st.hy_y);
        hx_ij = __ldg(a.Hx + oHx - 1 - st.hx_y);
        if (MAT) m2 = __ldg(a.mat + (unsigned)(i - 1) + (unsigned)(j - 1) * st.m_y + (unsigned)(k < nz ? k : nz - 1) * st.m_z);
    }
    CaCb<T> c0{1, 0}, c1{1, 0}, c2{1, 0};
    if (MAT) {
        if (ex) c0 = load_cab(a.cab + m0);
        if (ey) c1 = load_cab(a.cab + m1);
        if (ez) c2 = load_cab(a.cab + m2);
    }
    // ca E + cb c, or E + ce c without materials (ca = 1 multiplies exactly)
    auto upd = [&](T e, const CaCb<T> &m, T c) { return MAT ? radd(rmul(m.ca, e), rmul(m.cb, c)) : radd(e, rmul(a.ce, c)); };
    if (ex) {
        if (slab && (a.pe[1].on[j] | a.pe[2].on[k])) {
            T c = pml_curl(rsub(hz_k, hz_jk), rsub(hy_j, hy_jk), a.pe[1], j, a.pe[2], k, &a.psiE[0][0][px], &a.psiE[0][1][px]);
            a.Ex[px] = upd(ex0, c0, c);
        } else {
            a.Ex[px] = upd(ex0, c0, curl4(hz_k, hz_jk, hy_j, hy_jk));
        }
    }
    if (ey) {
        if (slab && (a.pe[2].on[k] | a.pe[0].on[i])) {
            T c = pml_curl(rsub(hx_i, hx_ik), rsub(hz_k, hz_ik), a.pe[2], k, a.pe[0], i, &a.psiE[1][0][py], &a.psiE[1][1][py]);
            a.Ey[py] = upd(ey0, c1, c);
        } else {
            a.Ey[py] = upd(ey0, c1, curl4(hx_i, hx_ik, hz_k, hz_ik));
        }
    }
    if (ez) {
        if (slab && (a.pe[0].on[i] | a.pe[1].on[j])) {
            T c = pml_curl(rsub(hy_j, hy_ij), rsub(hx_i, hx_ij), a.pe[0], i, a.pe[1], j, &a.psiE[2][0][pz], &a.psiE[2][1][pz]);
            a.Ez[pz] = upd(ez0, c2, c);
        } else {
            a.Ez[pz] = upd(ez0, c2, curl4(hy_j, hy_ij, hx_i, hx_ij));
        }
    }
}

template <class T, bool MAT, bool PML>
__global__ void __launch_bounds__(256) fdtd_e_kernel(FdtdArgs<T> a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i > a.nx || j > a.ny) return;
    const bool slab = PML && !block_outside_slabs(a);
#pragma unroll
    for (int kk = 0; kk < kFdtdKZ; ++kk) {
        const int k = blockIdx.z * kFdtdKZ + kk;
        if (k <= a.nz) fdtd_e_cell<T, MAT, PML>(a, i, j, k, slab);
    }
}

// ------------------------------------------------------------- fused step
// One pass per step: H^{n+1/2} and then E^{n+1} plane by plane along z.  A
// block owns a 31 x 7 tile of (i, j) columns and a chunk of kFusedKZ planes;
// its 32 x 8 threads also compute H on the tile's -x and -y halo columns
// (and the plane below the chunk), whose E update needs them, instead of
// waiting for the neighbouring blocks.  So every block reads only old
// values: E, H and the H-type CPML auxiliaries are double-buffered (read
// from the old copy, the owner writes the new one; halo values are formed
// and dropped), E's auxiliaries are read and written by their owner only.
// The new H of two planes sits in shared memory for the E update.  Per cell
// the arithmetic is that of fdtd_h_cell / fdtd_e_cell, so results are the
// bits of the two-kernel step.  Traffic: E and H read once, written once
// (12 words per cell) instead of 18.  Opt-in (EMS_FDTD_FUSED=1): on the
// 512^3 CPML workload the plane march, two barriers per plane, ran 3.42 ms
// per step against 2.39 ms for the two kernels, latency-bound at 4 blocks
// of 256 threads per SM.
constexpr int kFusedKZ = 32, kFusedBX = 32, kFusedBY = 8;

template <class T> struct FusedArgs {
    FdtdArgs<T> a;                  // old fields (Ex..Hz) and the shared data
    T *Exn, *Eyn, *Ezn, *Hxn, *Hyn, *Hzn;   // new fields
    T *psiHn[3][2];                 // new H-type CPML auxiliaries (a.psiH: the old ones)
};

// psi recursion with separate read and write copies (write == nullptr: form only)
template <class T>
__device__ __forceinline__ T pml_curl_rw(T d1, T d2, const Prof<T> &p1, int s1, const Prof<T> &p2, int s2, const T *r1,
                                         const T *r2, T *w1, T *w2)
{
    T q1 = radd(rmul(p1.b[s1], *r1), rmul(p1.a[s1], d1));
    T q2 = radd(rmul(p2.b[s2], *r2), rmul(p2.a[s2], d2));
    if (w1) { *w1 = q1; *w2 = q2; }
    return rsub(radd(rsub(rmul(p1.kinv[s1], d1), rmul(p2.kinv[s2], d2)), q1), q2);
}

template <class T, bool MAT, bool PML>
__global__ void __launch_bounds__(kFusedBX * kFusedBY, 4) fdtd_fused_kernel(FusedArgs<T> f)
{
    const FdtdArgs<T> &a = f.a;
    const FdtdStrides &st = a.st;
    __shared__ T sH[2][3][kFusedBY][kFusedBX];   // new H of planes k (parity) for the tile and its halo
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i = (int)blockIdx.x * (kFusedBX - 1) + tx - 1, j = (int)blockIdx.y * (kFusedBY - 1) + ty - 1;
    const int kb = (int)blockIdx.z * kFusedKZ, ke = min(kb + kFusedKZ, a.nz + 1);
    const bool col = i >= 0 && j >= 0 && i <= a.nx && j <= a.ny;   // an H column of the grid
    const bool own = col && tx > 0 && ty > 0;                       // a column of the tile (E and the stored H)
    bool slab = false;
    if (PML) {
        const int i0 = (int)blockIdx.x * (kFusedBX - 1) - 1, j0 = (int)blockIdx.y * (kFusedBY - 1) - 1;
        slab = !(i0 >= a.in_lo[0] && i0 + kFusedBX <= a.in_hi[0] && j0 >= a.in_lo[1] && j0 + kFusedBY <= a.in_hi[1] &&
                 kb - 1 >= a.in_lo[2] && ke <= a.in_hi[2]);
    }
    for (int k = max(kb - 1, 0); k < ke; ++k) {
        const int pk = k & 1;
        // ---- the E update's own loads (old E, material coefficients), issued
        // before the H update so that their latency overlaps it and the barrier
        const bool edo = own && k >= kb;
        const bool ex = edo && j >= 1 && k >= 1, ey = edo && i >= 1 && k >= 1, ez = edo && i >= 1 && j >= 1;
        const unsigned qx = i + j * st.ex_y + k * st.ex_z, qy = i + j * st.ey_y + k * st.ey_z;
        const unsigned qz = i + j * st.ez_y + k * st.ez_z;
        T ex0 = 0, ey0 = 0, ez0 = 0;
        CaCb<T> c0{1, 0}, c1{1, 0}, c2{1, 0};
        {
            const int nx = a.nx, ny = a.ny, nz = a.nz;
            unsigned m0 = 0, m1 = 0, m2 = 0;
            if (ex) {
                ex0 = __ldg(a.Ex + qx);
                if (MAT) m0 = __ldg(a.mat + (unsigned)(i < nx ? i : nx - 1) + (unsigned)(j - 1) * st.m_y + (unsigned)(k - 1) * st.m_z);
            }
            if (ey) {
                ey0 = __ldg(a.Ey + qy);
                if (MAT) m1 = __ldg(a.mat + (unsigned)(i - 1) + (unsigned)(j < ny ? j : ny - 1) * st.m_y + (unsigned)(k - 1) * st.m_z);
            }
            if (ez) {
                ez0 = __ldg(a.Ez + qz);
                if (MAT) m2 = __ldg(a.mat + (unsigned)(i - 1) + (unsigned)(j - 1) * st.m_y + (unsigned)(k < nz ? k : nz - 1) * st.m_z);
            }
            if (MAT) {
                if (ex) c0 = load_cab(a.cab + m0);
                if (ey) c1 = load_cab(a.cab + m1);
                if (ez) c2 = load_cab(a.cab + m2);
            }
        }
        // ---- H^{n+1/2} at (i, j, k) from the old E (fdtd_h_cell)
        T hxv = 0, hyv = 0, hzv = 0;
        if (col) {
            const bool store = own && k >= kb;
            const unsigned oEx = i + j * st.ex_y + k * st.ex_z, oEy = i + j * st.ey_y + k * st.ey_z;
            const unsigned oEz = i + j * st.ez_y + k * st.ez_z;
            const unsigned px = i + j * st.hx_y + k * st.hx_z, py = i + j * st.hy_y + k * st.hy_z;
            const unsigned pz = i + j * st.hz_y + k * st.hz_z;
            const bool hx = i < a.nx, hy = j < a.ny, hz = k < a.nz;
            T ez11 = 0, ey1k = 0, ex1k = 0, ez1 = 0, ey1 = 0, ex1 = 0, ez0 = 0, ey0 = 0, ex0 = 0, hx0 = 0, hy0 = 0, hz0 = 0;
            if (hx || hy) ez11 = __ldg(a.Ez + oEz + 1 + st.ez_y);
            if (hx || hz) ey1k = __ldg(a.Ey + oEy + 1 + st.ey_z);
            if (hy || hz) ex1k = __ldg(a.Ex + oEx + st.ex_y + st.ex_z);
            if (hx) { hx0 = __ldg(a.Hx + px); ez1 = __ldg(a.Ez + oEz + 1); ey1 = __ldg(a.Ey + oEy + 1); }
            if (hy) { hy0 = __ldg(a.Hy + py); ex1 = __ldg(a.Ex + oEx + st.ex_y); ez0 = __ldg(a.Ez + oEz + st.ez_y); }
            if (hz) { hz0 = __ldg(a.Hz + pz); ey0 = __ldg(a.Ey + oEy + st.ey_z); ex0 = __ldg(a.Ex + oEx + st.ex_z); }
            if (hx) {
                T c;
                if (PML && slab && (a.ph[1].on[j] | a.ph[2].on[k]))
                    c = pml_curl_rw(rsub(ez11, ez1), rsub(ey1k, ey1), a.ph[1], j, a.ph[2], k, &a.psiH[0][0][px], &a.psiH[0][1][px],
                                    store ? &f.psiHn[0][0][px] : nullptr, store ? &f.psiHn[0][1][px] : nullptr);
                else
                    c = curl4(ez11, ez1, ey1k, ey1);
                hxv = rsub(hx0, rmul(a.ch, c));
                if (store) f.Hxn[px] = hxv;
            }
            if (hy) {
                T c;
                if (PML && slab && (a.ph[2].on[k] | a.ph[0].on[i]))
                    c = pml_curl_rw(rsub(ex1k, ex1), rsub(ez11, ez0), a.ph[2], k, a.ph[0], i, &a.psiH[1][0][py], &a.psiH[1][1][py],
                                    store ? &f.psiHn[1][0][py] : nullptr, store ? &f.psiHn[1][1][py] : nullptr);
                else
                    c = curl4(ex1k, ex1, ez11, ez0);
                hyv = rsub(hy0, rmul(a.ch, c));
                if (store) f.Hyn[py] = hyv;
            }
            if (hz) {
                T c;
                if (PML && slab && (a.ph[0].on[i] | a.ph[1].on[j]))
                    c = pml_curl_rw(rsub(ey1k, ey0), rsub(ex1k, ex0), a.ph[0], i, a.ph[1], j, &a.psiH[2][0][pz], &a.psiH[2][1][pz],
                                    store ? &f.psiHn[2][0][pz] : nullptr, store ? &f.psiHn[2][1][pz] : nullptr);
                else
                    c = curl4(ey1k, ey0, ex1k, ex0);
                hzv = rsub(hz0, rmul(a.ch, c));
                if (store) f.Hzn[pz] = hzv;
            }
        }
        sH[pk][0][ty][tx] = hxv;
        sH[pk][1][ty][tx] = hyv;
        sH[pk][2][ty][tx] = hzv;
        __syncthreads();
        // ---- E^{n+1} at (i, j, k) from the new H (fdtd_e_cell)
        if (edo) {
            const int q = pk ^ 1;
            const unsigned px = qx, py = qy, pz = qz;
            // H(i,j,k-1), H(i,j-1,k), H(i-1,j,k) and the diagonal neighbours, from shared memory
            const T hz_k = sH[q][2][ty][tx], hy_j = sH[pk][1][ty - 1][tx], hx_i = sH[pk][0][ty][tx - 1];
            const T hz_jk = sH[q][2][ty - 1][tx], hy_jk = sH[q][1][ty - 1][tx];
            const T hx_ik = sH[q][0][ty][tx - 1], hz_ik = sH[q][2][ty][tx - 1];
            const T hy_ij = sH[pk][1][ty - 1][tx - 1], hx_ij = sH[pk][0][ty - 1][tx - 1];
            auto upd = [&](T e, const CaCb<T> &m, T c) { return MAT ? radd(rmul(m.ca, e), rmul(m.cb, c)) : radd(e, rmul(a.ce, c)); };
            if (ex) {
                T c;
                if (PML && slab && (a.pe[1].on[j] | a.pe[2].on[k]))
                    c = pml_curl(rsub(hz_k, hz_jk), rsub(hy_j, hy_jk), a.pe[1], j, a.pe[2], k, &a.psiE[0][0][px], &a.psiE[0][1][px]);
                else
                    c = curl4(hz_k, hz_jk, hy_j, hy_jk);
                f.Exn[px] = upd(ex0, c0, c);
            }
            if (ey) {
                T c;
                if (PML && slab && (a.pe[2].on[k] | a.pe[0].on[i]))
                    c = pml_curl(rsub(hx_i, hx_ik), rsub(hz_k, hz_ik), a.pe[2], k, a.pe[0], i, &a.psiE[1][0][py], &a.psiE[1][1][py]);
                else
                    c = curl4(hx_i, hx_ik, hz_k, hz_ik);
                f.Eyn[py] = upd(ey0, c1, c);
            }
            if (ez) {
                T c;
                if (PML && slab && (a.pe[0].on[i] | a.pe[1].on[j]))
                    c = pml_curl(rsub(hy_j, hy_ij), rsub(hx_i, hx_ij), a.pe[0], i, a.pe[1], j, &a.psiE[2][0][pz], &a.psiE[2][1][pz]);
                else
                    c = curl4(hy_j, hy_ij, hx_i, hx_ij);
                f.Ezn[pz] = upd(ez0, c2, c);
            }
        }
        __syncthreads();
    }
}

// Point sources in insertion order: E[src] -= v (fdtd_simulation.cpp:222-239).
template <class T>
__global__ void fdtd_source_kernel(T *Ex, T *Ey, T *Ez, const int *comp, const size_t *off, const double *vals, int nsrc)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int s = 0; s < nsrc; ++s) {
        T *f = comp[s] == 0 ? Ex : comp[s] == 1 ? Ey : Ez;
        f[off[s]] = rsub(f[off[s]], (T)vals[s]);
    }
}

// Receiver averages (fdtd_simulation.cpp:261-303): one thread per receiver,
// summing its listed samples in order, then dividing by the count.
template <class T>
__global__ void fdtd_receiver_kernel(const T *Ex, const T *Ey, const T *Ez, int nobs, const int *cnt,
                                     const int *start, const size_t *off, double *trace_row, int nsamp)
{
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nobs) return;
    double *out = trace_row + (size_t)o * nsamp * 3;
    int q = start[o];
    for (int c = 0; c < 3; ++c) {
        const T *f = c == 0 ? Ex : c == 1 ? Ey : Ez;
        int n = cnt[3 * o + c];
        double acc = out[c];
        for (int r = 0; r < n; ++r, ++q) acc = __dadd_rn(acc, (double)f[off[q]]);
        out[c] = acc / (double)n;
    }
}

double fdtd_source_value(int kind, double f0, double t, double h)
{
    if (kind == EMS_WAVE_REFERENCE)
        return -4.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) *
               std::exp(-2.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) * (t - 1.0 / f0)) / h / h / h * 0.001;
    double tau = t - std::sqrt(2.0) / f0;
    return (1.0 - 2.0 * M_PI * M_PI * f0 * f0 * tau * tau) * std::exp(-M_PI * M_PI * f0 * f0 * tau * tau) / h / h / h * 0.001;
}

struct FdtdSource {
    int comp;
    int ijk[3];
    int kind;
    double f0, amp;
    size_t off;
};

struct FdtdSim : Sim {
    ems_fdtd_params P;
    int nx, ny, nz;
    bool fp64;
    size_t n[6];
    DevBuf F[6];
    DevBuf G[6];                // the other copy of the fields (the fused step writes it; swapped after each step)
    bool fused = false;         // one fused H+E pass per step (EMS_FDTD_FUSED=1; default: the H and E kernels)
    // materials
    std::vector<uint16_t> mat_host;
    std::vector<double> mat_eps, mat_sigma;
    DevBuf d_mat, d_cab;
    // CPML
    DevBuf d_prof[2][3][4];   // [E/H][axis][b,a,kinv,on]
    std::vector<unsigned char> pml_on[2][3];   // host copies of the "on" flags
    DevBuf d_psiE[3][2], d_psiH[3][2], d_psiH2[3][2];
    // sources, receivers
    std::vector<FdtdSource> srcs;
    std::vector<std::vector<std::array<int, 3>>> obs_lists;   // 3 per receiver
    std::vector<int> obs_n;
    DevBuf d_src_comp, d_src_off, d_src_vals, d_obs_cnt, d_obs_start, d_obs_off, d_traces;
    bool dirty = true;

    explicit FdtdSim(const ems_fdtd_params *p) : Sim(Kind::FDTD), P(*p)
    {
        nx = P.grid[0]; ny = P.grid[1]; nz = P.grid[2];
        EMS_CHECK_ARG(nx > 0 && ny > 0 && nz > 0, "grid sizes must be positive");
        EMS_CHECK_ARG((double)(nx + 2) * (ny + 2) * (nz + 2) < 4294967296.0, "grid too large for 32-bit array offsets");
        EMS_CHECK_ARG(P.h > 0 && P.dt > 0 && P.permittivity > 0 && P.permeability > 0, "h, dt, eps, mu must be positive");
        EMS_CHECK_ARG(P.time_frequency > 0, "time_frequency must be positive");
        EMS_CHECK_ARG(P.precision == EMS_FP64 || P.precision == EMS_FP32, "precision must be EMS_FP64 or EMS_FP32");
        // the reference's check_params condition (fdtd_simulation.cpp:358): c*dt < h
        double c = 1.0 / std::sqrt(P.permittivity * P.permeability);
        EMS_CHECK_ARG(c * P.dt < P.h, "time step violates c*dt < h (reference check_params)");
        EMS_CHECK_ARG(P.pml_cells >= 0 && 2 * P.pml_cells < std::min(nx, std::min(ny, nz)), "pml_cells too large for the grid");
        if (P.pml_order == 0) P.pml_order = 3.0;
        if (P.pml_kappa_max == 0) P.pml_kappa_max = 1.0;
        if (P.pml_reflection == 0) P.pml_reflection = 1e-6;
        fp64 = P.precision == EMS_FP64;
        n[0] = (size_t)(nx + 1) * (ny + 2) * (nz + 2);
        n[1] = (size_t)(nx + 2) * (ny + 1) * (nz + 2);
        n[2] = (size_t)(nx + 2) * (ny + 2) * (nz + 1);
        n[3] = (size_t)nx * (ny + 1) * (nz + 1);
        n[4] = (size_t)(nx + 1) * ny * (nz + 1);
        n[5] = (size_t)(nx + 1) * (ny + 1) * nz;
        init_stream();
        size_t w = fp64 ? 8 : 4;
        if (const char *env = std::getenv("EMS_FDTD_FUSED")) fused = std::strcmp(env, "1") == 0;
        for (int q = 0; q < 6; ++q) { F[q].alloc(n[q] * w); F[q].zero(stream); }
        if (fused)
            for (int q = 0; q < 6; ++q) { G[q].alloc(n[q] * w); G[q].zero(stream); }
        if (P.pml_cells > 0) setup_pml();
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    void setup_pml()
    {
        const int nn[3] = {nx, ny, nz};
        const int L = P.pml_cells;
        double eta = std::sqrt(P.permeability / P.permittivity);
        double smax = -(P.pml_order + 1.0) * std::log(P.pml_reflection) / (2.0 * eta * L * P.h);
        for (int eh = 0; eh < 2; ++eh)
            for (int d = 0; d < 3; ++d) {
                int cnt = nn[d] + 2;
                std::vector<double> b(cnt, 0.0), av(cnt, 0.0), kinv(cnt, 1.0);
                std::vector<unsigned char> on(cnt, 0);
                double shift = eh == 0 ? -0.5 : 0.0;
                for (int s = 0; s < cnt; ++s) {
                    double x = s + shift, lo = L - x, hi = x - (nn[d] - L);
                    double dd = lo > hi ? lo : hi;
                    dd = dd < 0.0 ? 0.0 : (dd > L ? 1.0 : dd / L);
                    if (dd <= 0.0) continue;
                    double g = std::pow(dd, P.pml_order);
                    double sig = smax * g, kap = 1.0 + (P.pml_kappa_max - 1.0) * g, alp = P.pml_alpha_max * (1.0 - dd);
                    double bb = std::exp(-(sig / kap + alp) * P.dt / P.permittivity);
                    b[s] = bb;
                    av[s] = sig > 0.0 ? sig / (sig * kap + kap * kap * alp) * (bb - 1.0) : 0.0;
                    kinv[s] = 1.0 / kap;
                    on[s] = 1;
                }
                upload_real(d_prof[eh][d][0], b);
                upload_real(d_prof[eh][d][1], av);
                upload_real(d_prof[eh][d][2], kinv);
                d_prof[eh][d][3].alloc(cnt);
                EMS_CUDA(cudaMemcpyAsync(d_prof[eh][d][3].p, on.data(), cnt, cudaMemcpyHostToDevice, stream));
                pml_on[eh][d] = on;
            }
        size_t w = fp64 ? 8 : 4;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 2; ++r) {
                d_psiE[c][r].alloc(n[c] * w); d_psiE[c][r].zero(stream);
                d_psiH[c][r].alloc(n[3 + c] * w); d_psiH[c][r].zero(stream);
                if (fused) { d_psiH2[c][r].alloc(n[3 + c] * w); d_psiH2[c][r].zero(stream); }
            }
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    void upload_real(DevBuf &d, const std::vector<double> &v)
    {
        if (fp64) {
            d.alloc(v.size() * 8);
            EMS_CUDA(cudaMemcpyAsync(d.p, v.data(), v.size() * 8, cudaMemcpyHostToDevice, stream));
        } else {
            std::vector<float> f(v.begin(), v.end());
            d.alloc(f.size() * 4);
            EMS_CUDA(cudaMemcpyAsync(d.p, f.data(), f.size() * 4, cudaMemcpyHostToDevice, stream));
        }
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    size_t ex_index(int c, const int *q) const
    {
        if (c == 0) return (size_t)q[0] + (size_t)q[1] * (nx + 1) + (size_t)q[2] * (nx + 1) * (ny + 2);
        if (c == 1) return (size_t)q[0] + (size_t)q[1] * (nx + 2) + (size_t)q[2] * (nx + 2) * (ny + 1);
        return (size_t)q[0] + (size_t)q[1] * (nx + 2) + (size_t)q[2] * (nx + 2) * (ny + 2);
    }
    bool in_e(int c, const int *q) const
    {
        int lim[3][3] = {{nx, ny + 1, nz + 1}, {nx + 1, ny, nz + 1}, {nx + 1, ny + 1, nz}};
        for (int d = 0; d < 3; ++d)
            if (q[d] < 0 || q[d] > lim[c][d]) return false;
        return true;
    }

    void set_material(const double *eps, const double *sigma)
    {
        EMS_CHECK_ARG(eps != nullptr, "eps array required");
        size_t nc = (size_t)nx * ny * nz;
        std::map<std::pair<double, double>, int> ids;
        mat_host.assign(nc, 0);
        mat_eps.clear(); mat_sigma.clear();
        double last_e = -1.0, last_s = -1.0;
        int last_id = -1;
        for (size_t q = 0; q < nc; ++q) {
            double e = eps[q], s = sigma ? sigma[q] : 0.0;
            if (e == last_e && s == last_s) {   // runs of equal material along x
                mat_host[q] = (uint16_t)last_id;
                continue;
            }
            EMS_CHECK_ARG(std::isfinite(e) && e > 0 && std::isfinite(s) && s >= 0, "eps must be > 0 and sigma >= 0");
            auto key = std::make_pair(e, s);
            auto it = ids.find(key);
            int id;
            if (it == ids.end()) {
                EMS_CHECK_ARG(ids.size() < 65535, "more than 65535 distinct (eps, sigma) pairs");
                id = (int)ids.size();
                ids.emplace(key, id);
                mat_eps.push_back(e); mat_sigma.push_back(s);
            } else {
                id = it->second;
            }
            mat_host[q] = (uint16_t)id;
            last_e = e; last_s = s; last_id = id;
        }
        std::vector<double> ca(mat_eps.size()), cb(mat_eps.size());
        for (size_t m = 0; m < mat_eps.size(); ++m) {
            double s = mat_sigma[m] * P.dt / (2.0 * mat_eps[m]);
            ca[m] = (1.0 - s) / (1.0 + s);
            cb[m] = P.dt / mat_eps[m] / P.h / (1.0 + s);
        }
        d_mat.alloc(nc * 2);
        EMS_CUDA(cudaMemcpyAsync(d_mat.p, mat_host.data(), nc * 2, cudaMemcpyHostToDevice, stream));
        std::vector<double> cab(2 * ca.size());
        for (size_t m = 0; m < ca.size(); ++m) { cab[2 * m] = ca[m]; cab[2 * m + 1] = cb[m]; }
        upload_real(d_cab, cab);
    }

    template <class T> FdtdArgs<T> args() const
    {
        FdtdArgs<T> a{};
        a.Ex = F[0].as<T>(); a.Ey = F[1].as<T>(); a.Ez = F[2].as<T>();
        a.Hx = F[3].as<T>(); a.Hy = F[4].as<T>(); a.Hz = F[5].as<T>();
        a.nx = nx; a.ny = ny; a.nz = nz;
        const unsigned X = nx, Y = ny;
        a.st = FdtdStrides{X + 1, (X + 1) * (Y + 2), X + 2, (X + 2) * (Y + 1), X + 2, (X + 2) * (Y + 2),
                           X, X * (Y + 1), X + 1, (X + 1) * Y, X + 1, (X + 1) * (Y + 1), X, X * Y};
        a.ch = (T)(P.dt / P.permeability / P.h);
        a.ce = (T)(P.dt / P.permittivity / P.h);
        a.mat = d_mat.as<uint16_t>();
        a.cab = d_cab.as<CaCb<T>>();
        if (P.pml_cells > 0)
            for (int d = 0; d < 3; ++d) {
                // the index range between the slabs, where neither profile is on
                const auto &oe = pml_on[0][d], &oh = pml_on[1][d];
                int lo = 0, hi = (int)oe.size();
                while (lo < hi && (oe[lo] | oh[lo])) ++lo;
                while (hi > lo && (oe[hi - 1] | oh[hi - 1])) --hi;
                for (int q = lo; q < hi; ++q)
                    if (oe[q] | oh[q]) throw Error{EMS_ERR_STATE, "CPML profile is not two slabs"};
                a.in_lo[d] = lo;
                a.in_hi[d] = hi;
                a.pe[d] = Prof<T>{d_prof[0][d][0].as<T>(), d_prof[0][d][1].as<T>(), d_prof[0][d][2].as<T>(), d_prof[0][d][3].as<unsigned char>()};
                a.ph[d] = Prof<T>{d_prof[1][d][0].as<T>(), d_prof[1][d][1].as<T>(), d_prof[1][d][2].as<T>(), d_prof[1][d][3].as<unsigned char>()};
                for (int r = 0; r < 2; ++r) { a.psiE[d][r] = d_psiE[d][r].as<T>(); a.psiH[d][r] = d_psiH[d][r].as<T>(); }
            }
        return a;
    }

    // Launch shape of the H and E kernels (x, y threads; one z plane per
    // block row), chosen by tune_shape on the handle's first run of at least
    // kTuneMinSteps steps.  Every cell is one thread whatever the shape, so
    // the shape changes no result.
    dim3 blk{32, 8, 1};
    bool tuned = false;
    dim3 block() const { return blk; }
    void launch_shape(int b[3]) override { b[0] = (int)blk.x; b[1] = (int)blk.y; b[2] = 1; }
    dim3 grid() const
    {
        return dim3((nx + 1 + blk.x - 1) / blk.x, (ny + 1 + blk.y - 1) / blk.y, (nz + 1 + kFdtdKZ - 1) / kFdtdKZ);
    }

    static constexpr int kShapes = 6, kTuneSteps = 3, kTuneMinSteps = 24;
    static constexpr unsigned kShape[kShapes][2] = {{32, 8}, {32, 4}, {64, 4}, {128, 2}, {256, 1}, {64, 2}};

    // Steps of this run spent tuning: the environment variable
    // EMS_FDTD_BLOCK="XxY" forces one of the shapes; otherwise the first run
    // of at least kTuneMinSteps steps advances kTuneSteps steps with each
    // shape (one warm-up, two timed) and keeps the fastest.
    int tune_steps(int nsteps)
    {
        if (tuned) return 0;
        if (const char *env = std::getenv("EMS_FDTD_BLOCK")) {
            unsigned x = 0, y = 0;
            if (std::sscanf(env, "%ux%u", &x, &y) == 2)
                for (auto &sh : kShape)
                    if (sh[0] == x && sh[1] == y) { blk = dim3(x, y, 1); tuned = true; return 0; }
            throw Error{EMS_ERR_INVALID_ARGUMENT, "EMS_FDTD_BLOCK must be one of 32x8 32x4 64x4 128x2 256x1 64x2"};
        }
        return nsteps >= kTuneMinSteps ? kShapes * kTuneSteps : 0;
    }

    template <class T> void launch_h(const FdtdArgs<T> &a)
    {
        if (P.pml_cells > 0) fdtd_h_kernel<T, true><<<grid(), block(), 0, stream>>>(a);
        else fdtd_h_kernel<T, false><<<grid(), block(), 0, stream>>>(a);
    }
    // The fused step: reads F (and the old H auxiliaries), writes G (and the
    // new ones), then the copies are swapped.
    template <class T> void launch_fused(const FdtdArgs<T> &a)
    {
        FusedArgs<T> f;
        f.a = a;
        f.Exn = G[0].as<T>(); f.Eyn = G[1].as<T>(); f.Ezn = G[2].as<T>();
        f.Hxn = G[3].as<T>(); f.Hyn = G[4].as<T>(); f.Hzn = G[5].as<T>();
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 2; ++r) f.psiHn[c][r] = P.pml_cells > 0 ? d_psiH2[c][r].as<T>() : nullptr;
        const dim3 blk(kFusedBX, kFusedBY, 1);
        const dim3 grd((nx + 1 + kFusedBX - 2) / (kFusedBX - 1), (ny + 1 + kFusedBY - 2) / (kFusedBY - 1),
                       (nz + 1 + kFusedKZ - 1) / kFusedKZ);
        const bool mat = !mat_host.empty(), pml = P.pml_cells > 0;
        if (mat && pml) fdtd_fused_kernel<T, true, true><<<grd, blk, 0, stream>>>(f);
        else if (mat) fdtd_fused_kernel<T, true, false><<<grd, blk, 0, stream>>>(f);
        else if (pml) fdtd_fused_kernel<T, false, true><<<grd, blk, 0, stream>>>(f);
        else fdtd_fused_kernel<T, false, false><<<grd, blk, 0, stream>>>(f);
    }
    void swap_copies()
    {
        for (int q = 0; q < 6; ++q) std::swap(F[q].p, G[q].p);
        if (P.pml_cells > 0)
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 2; ++r) std::swap(d_psiH[c][r].p, d_psiH2[c][r].p);
    }
    template <class T> void launch_e(const FdtdArgs<T> &a)
    {
        bool mat = !mat_host.empty(), pml = P.pml_cells > 0;
        if (mat && pml) fdtd_e_kernel<T, true, true><<<grid(), block(), 0, stream>>>(a);
        else if (mat) fdtd_e_kernel<T, true, false><<<grid(), block(), 0, stream>>>(a);
        else if (pml) fdtd_e_kernel<T, false, true><<<grid(), block(), 0, stream>>>(a);
        else fdtd_e_kernel<T, false, false><<<grid(), block(), 0, stream>>>(a);
    }

    template <class T> void run_t(int nsteps)
    {
        const int tf = P.time_frequency;
        nsamp = nsteps / tf + 1;
        nobs = (int)obs_n.size() / 3;
        ncols = 3;
        // source values per step, computed on the host in FP64 exactly as the
        // reference does (time accumulated by repeated addition of dt)
        int ns = (int)srcs.size();
        std::vector<double> vals((size_t)std::max(ns, 1) * nsteps, 0.0);
        double t = 0.0;
        for (int st = 0; st < nsteps; ++st) {
            for (int s = 0; s < ns; ++s) {
                const FdtdSource &q = srcs[s];
                double eps = P.permittivity, div = 1.0;
                if (!mat_host.empty()) {
                    int ci = q.ijk[0], cj = q.ijk[1], ck = q.ijk[2];
                    if (q.comp == 0) { ci = ci < nx ? ci : nx - 1; cj -= 1; ck -= 1; }
                    else if (q.comp == 1) { ci -= 1; cj = cj < ny ? cj : ny - 1; ck -= 1; }
                    else { ci -= 1; cj -= 1; ck = ck < nz ? ck : nz - 1; }
                    int m = mat_host[(size_t)ci + (size_t)cj * nx + (size_t)ck * nx * ny];
                    eps = mat_eps[m];
                    div = 1.0 + mat_sigma[m] * P.dt / (2.0 * mat_eps[m]);
                }
                double v = fdtd_source_value(q.kind, q.f0, t, P.h) * q.amp * P.dt / eps;
                if (div != 1.0) v /= div;
                vals[(size_t)st * ns + s] = v;
            }
            t += P.dt;
        }
        std::vector<int> comp(std::max(ns, 1));
        std::vector<size_t> off(std::max(ns, 1));
        for (int s = 0; s < ns; ++s) { comp[s] = srcs[s].comp; off[s] = srcs[s].off; }
        d_src_comp.alloc(comp.size() * 4); d_src_off.alloc(off.size() * 8); d_src_vals.alloc(vals.size() * 8);
        EMS_CUDA(cudaMemcpyAsync(d_src_comp.p, comp.data(), comp.size() * 4, cudaMemcpyHostToDevice, stream));
        EMS_CUDA(cudaMemcpyAsync(d_src_off.p, off.data(), off.size() * 8, cudaMemcpyHostToDevice, stream));
        EMS_CUDA(cudaMemcpyAsync(d_src_vals.p, vals.data(), vals.size() * 8, cudaMemcpyHostToDevice, stream));
        // receivers
        std::vector<int> start(std::max(nobs, 1), 0);
        std::vector<size_t> roff;
        for (int o = 0; o < nobs; ++o) {
            start[o] = (int)roff.size();
            for (int c = 0; c < 3; ++c)
                for (auto &q : obs_lists[3 * o + c]) roff.push_back(ex_index(c, q.data()));
        }
        if (roff.empty()) roff.push_back(0);
        d_obs_cnt.alloc(std::max<size_t>(obs_n.size(), 1) * 4);
        d_obs_start.alloc(start.size() * 4);
        d_obs_off.alloc(roff.size() * 8);
        if (!obs_n.empty()) EMS_CUDA(cudaMemcpyAsync(d_obs_cnt.p, obs_n.data(), obs_n.size() * 4, cudaMemcpyHostToDevice, stream));
        EMS_CUDA(cudaMemcpyAsync(d_obs_start.p, start.data(), start.size() * 4, cudaMemcpyHostToDevice, stream));
        EMS_CUDA(cudaMemcpyAsync(d_obs_off.p, roff.data(), roff.size() * 8, cudaMemcpyHostToDevice, stream));
        size_t ntr = (size_t)std::max(nobs, 1) * nsamp * 3;
        d_traces.alloc(ntr * 8);
        d_traces.zero(stream);

        FdtdArgs<T> a = args<T>();
        long long launches = 0;
        const int tune = fused ? 0 : tune_steps(nsteps);
        struct TuneEvents {   // destroyed on every exit path
            cudaEvent_t e[2 * kShapes] = {};
            ~TuneEvents()
            {
                for (cudaEvent_t x : e)
                    if (x) cudaEventDestroy(x);
            }
        } tev;
        if (tune)
            for (cudaEvent_t &x : tev.e) EMS_CUDA(cudaEventCreate(&x));
        EMS_CUDA(cudaEventRecord(ev0, stream));
        for (int step = 1; step < nsteps + 1; ++step) {
            const int ts = step - 1, c = ts / kTuneSteps, r = ts % kTuneSteps;
            if (ts < tune) {
                blk = dim3(kShape[c][0], kShape[c][1], 1);
                if (r == 1) EMS_CUDA(cudaEventRecord(tev.e[2 * c], stream));
            }
            if (fused) {
                launch_fused<T>(a);
                swap_copies();
                a = args<T>();
                launches += 1;
            } else {
                launch_h<T>(a);
                launch_e<T>(a);
                launches += 2;
            }
            if (ns > 0) {
                fdtd_source_kernel<T><<<1, 32, 0, stream>>>(a.Ex, a.Ey, a.Ez, d_src_comp.as<int>(), d_src_off.as<size_t>(),
                                                           d_src_vals.as<double>() + (size_t)(step - 1) * ns, ns);
                ++launches;
            }
            if (nobs > 0 && step % tf == 0) {
                fdtd_receiver_kernel<T><<<(nobs + 127) / 128, 128, 0, stream>>>(
                    a.Ex, a.Ey, a.Ez, nobs, d_obs_cnt.as<int>(), d_obs_start.as<int>(), d_obs_off.as<size_t>(),
                    d_traces.as<double>() + (size_t)(step / tf) * 3, nsamp);
                ++launches;
            }
            if (ts < tune && r == kTuneSteps - 1) EMS_CUDA(cudaEventRecord(tev.e[2 * c + 1], stream));
            if (tune && step == tune) {   // all shapes timed: keep the fastest
                EMS_CUDA(cudaEventSynchronize(tev.e[2 * kShapes - 1]));
                float best = 0.0f;
                int pick = 0;
                for (int k = 0; k < kShapes; ++k) {
                    float ms = 0.0f;
                    EMS_CUDA(cudaEventElapsedTime(&ms, tev.e[2 * k], tev.e[2 * k + 1]));
                    if (k == 0 || ms < best) { best = ms; pick = k; }
                }
                blk = dim3(kShape[pick][0], kShape[pick][1], 1);
                tuned = true;
            }
        }
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaEventRecord(ev1, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        float ms = 0;
        EMS_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        last_ms = ms;
        last_launches = launches;
        traces.assign(ntr, 0.0);
        EMS_CUDA(cudaMemcpy(traces.data(), d_traces.p, ntr * 8, cudaMemcpyDeviceToHost));
        traces.resize((size_t)nobs * nsamp * 3);
    }

    void run(int nsteps) override
    {
        EMS_CHECK_ARG(nsteps >= 0, "num_steps must be >= 0");
        if (fp64) run_t<double>(nsteps); else run_t<float>(nsteps);
        check_finite({{F[0].p, n[0]}, {F[1].p, n[1]}, {F[2].p, n[2]}, {F[3].p, n[3]}, {F[4].p, n[4]}, {F[5].p, n[5]}}, fp64);
    }

    size_t field_size(int which) const override
    {
        if (which < 0 || which > 5) throw Error{EMS_ERR_INVALID_ARGUMENT, "field index must be 0..5 (Ex,Ey,Ez,Hx,Hy,Hz)"};
        return n[which];
    }
    void get_field(int which, double *out) const override
    {
        size_t cnt = field_size(which);
        if (fp64) {
            EMS_CUDA(cudaMemcpy(out, F[which].p, cnt * 8, cudaMemcpyDeviceToHost));
        } else {
            std::vector<float> tmp(cnt);
            EMS_CUDA(cudaMemcpy(tmp.data(), F[which].p, cnt * 4, cudaMemcpyDeviceToHost));
            for (size_t q = 0; q < cnt; ++q) out[q] = tmp[q];
        }
    }
    void set_field(int which, const double *in) override
    {
        size_t cnt = field_size(which);
        if (fp64) {
            EMS_CUDA(cudaMemcpy(F[which].p, in, cnt * 8, cudaMemcpyHostToDevice));
        } else {
            std::vector<float> tmp(in, in + cnt);
            EMS_CUDA(cudaMemcpy(F[which].p, tmp.data(), cnt * 4, cudaMemcpyHostToDevice));
        }
        // the fused step never writes the boundary values of the other copy: keep them equal
        if (fused) EMS_CUDA(cudaMemcpy(G[which].p, F[which].p, F[which].bytes, cudaMemcpyDeviceToDevice));
    }

    // fdtd_simulation.cpp:308-331: results_<i>_<dt>_<h>_<N>.csv in `path`
    // (a directory; "." if empty), default stream precision, columns
    // time,Ex,Ey,Ez with time = j*tf*dt.
    void save(const char *path) const override
    {
        std::string dir = (path && *path) ? path : ".";
        int nsteps_run = (nsamp - 1) * P.time_frequency;
        for (int o = 0; o < nobs; ++o) {
            std::string fn = dir + "/results_" + std::to_string(o) + "_" + std::to_string(P.dt) + "_" +
                             std::to_string(P.h) + "_" + std::to_string(nsteps_run) + ".csv";
            std::ofstream f(fn);
            if (!f.is_open()) throw Error{EMS_ERR_IO, "cannot open " + fn};
            f << "time,Ex,Ey,Ez" << std::endl;
            for (int j = 0; j < nsamp; ++j) {
                const double *r = &traces[((size_t)o * nsamp + j) * 3];
                f << j * P.time_frequency * P.dt << "," << r[0] << "," << r[1] << "," << r[2] << std::endl;
            }
        }
    }

    double sample_time(int j) const override { return j * P.time_frequency * P.dt; }

    void reset() override
    {
        for (int q = 0; q < 6; ++q) F[q].zero(stream);
        if (fused)
            for (int q = 0; q < 6; ++q) G[q].zero(stream);
        if (P.pml_cells > 0)
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 2; ++r) {
                    d_psiE[c][r].zero(stream); d_psiH[c][r].zero(stream);
                    if (fused) d_psiH2[c][r].zero(stream);
                }
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    // E points whose update runs the CPML recursion (two psi values each).
    double pml_e_points() const
    {
        if (P.pml_cells <= 0) return 0.0;
        auto pairs = [&](int d1, int n1, int d2, int n2) {
            double c = 0.0;
            for (int a = 1; a <= n1; ++a)
                for (int b = 1; b <= n2; ++b) c += (pml_on[0][d1][a] | pml_on[0][d2][b]) ? 1.0 : 0.0;
            return c;
        };
        return (nx + 1.0) * pairs(1, ny, 2, nz) + (ny + 1.0) * pairs(2, nz, 0, nx) + (nz + 1.0) * pairs(0, nx, 1, ny);
    }

    // H-type points whose update runs the CPML recursion (two psi values each).
    double pml_h_points() const
    {
        if (P.pml_cells <= 0) return 0.0;
        auto pairs = [&](int d1, int n1, int d2, int n2) {
            double c = 0.0;
            for (int a = 0; a <= n1; ++a)
                for (int b = 0; b <= n2; ++b) c += (pml_on[1][d1][a] | pml_on[1][d2][b]) ? 1.0 : 0.0;
            return c;
        };
        return (double)nx * pairs(1, ny, 2, nz) + (double)ny * pairs(2, nz, 0, nx) + (double)nz * pairs(0, nx, 1, ny);
    }

    void time_dominant(int launches, double *ms, double *bytes, std::string *name) override
    {
        size_t w = fp64 ? 8 : 4;
        size_t cells = (size_t)nx * ny * nz;
        const double matb = mat_host.empty() ? 0.0 : 2.0 * cells;
        if (fused) {
            // the fused step: E and H read and written once (12 words per
            // cell), the material id, two psi values read and written per
            // CPML point of either type.  It reads F and writes G (and the
            // new H auxiliaries); E's auxiliaries change in place, so they
            // are kept and put back.
            double b = (double)cells * 12.0 * w + matb + (pml_e_points() + pml_h_points()) * 4.0 * w;
            DevBuf save[6];
            if (P.pml_cells > 0)
                for (int c = 0; c < 3; ++c)
                    for (int r = 0; r < 2; ++r) {
                        DevBuf &sv = save[2 * c + r];
                        sv.alloc(d_psiE[c][r].bytes);
                        EMS_CUDA(cudaMemcpyAsync(sv.p, d_psiE[c][r].p, d_psiE[c][r].bytes, cudaMemcpyDeviceToDevice, stream));
                    }
            float t = 0;
            auto body = [&](auto tag) {
                using T = decltype(tag);
                auto a = args<T>();
                launch_fused<T>(a);
                EMS_CUDA(cudaEventRecord(ev0, stream));
                for (int r = 0; r < launches; ++r) launch_fused<T>(a);
                EMS_CUDA(cudaEventRecord(ev1, stream));
            };
            if (fp64) body(double()); else body(float());
            EMS_CUDA(cudaStreamSynchronize(stream));
            EMS_CUDA(cudaEventElapsedTime(&t, ev0, ev1));
            if (P.pml_cells > 0) {
                size_t q = 0;
                for (int c = 0; c < 3; ++c)
                    for (int r = 0; r < 2; ++r, ++q)
                        EMS_CUDA(cudaMemcpyAsync(d_psiE[c][r].p, save[q].p, d_psiE[c][r].bytes, cudaMemcpyDeviceToDevice, stream));
            }
            EMS_CUDA(cudaStreamSynchronize(stream));
            *ms = t / launches;
            *bytes = b;
            *name = fp64 ? "fdtd_fused_kernel<double>" : "fdtd_fused_kernel<float>";
            return;
        }
        // E update: reads H (3), reads and writes E (3), the material id, and
        // reads and writes two psi values per point inside the CPML
        double b = (double)cells * 9.0 * w + matb + pml_e_points() * 4.0 * w;
        std::vector<DevBuf> save(3);
        for (int q = 0; q < 3; ++q) {
            save[q].alloc(F[q].bytes);
            EMS_CUDA(cudaMemcpyAsync(save[q].p, F[q].p, F[q].bytes, cudaMemcpyDeviceToDevice, stream));
        }
        float t = 0;
        if (fp64) { auto a = args<double>(); launch_e<double>(a); EMS_CUDA(cudaEventRecord(ev0, stream)); for (int r = 0; r < launches; ++r) launch_e<double>(a); }
        else { auto a = args<float>(); launch_e<float>(a); EMS_CUDA(cudaEventRecord(ev0, stream)); for (int r = 0; r < launches; ++r) launch_e<float>(a); }
        EMS_CUDA(cudaEventRecord(ev1, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        EMS_CUDA(cudaEventElapsedTime(&t, ev0, ev1));
        for (int q = 0; q < 3; ++q)
            EMS_CUDA(cudaMemcpyAsync(F[q].p, save[q].p, F[q].bytes, cudaMemcpyDeviceToDevice, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        *ms = t / launches;
        *bytes = b;
        *name = fp64 ? "fdtd_e_kernel<double>" : "fdtd_e_kernel<float>";
    }
};

Sim *make_fdtd(const ems_fdtd_params *p) { return new FdtdSim(p); }

void fdtd_set_source(Sim *s, int comp, const int ijk[3], int waveform, double f0, double amp)
{
    auto *f = static_cast<FdtdSim *>(s);
    EMS_CHECK_ARG(comp >= 0 && comp < 3, "component must be 0, 1 or 2");
    EMS_CHECK_ARG(ijk != nullptr && f->in_e(comp, ijk), "source index outside the field array");
    EMS_CHECK_ARG(waveform == EMS_WAVE_REFERENCE || waveform == EMS_WAVE_RICKER, "unknown waveform");
    EMS_CHECK_ARG(f0 > 0 && std::isfinite(amp), "f0 must be positive");
    FdtdSource q{comp, {ijk[0], ijk[1], ijk[2]}, waveform, f0, amp, f->ex_index(comp, ijk)};
    f->srcs.push_back(q);
}

void fdtd_add_observation(Sim *s, const int *x, int nx_, const int *y, int ny_, const int *z, int nz_)
{
    auto *f = static_cast<FdtdSim *>(s);
    const int *lists[3] = {x, y, z};
    int cnt[3] = {nx_, ny_, nz_};
    for (int c = 0; c < 3; ++c) {
        EMS_CHECK_ARG(cnt[c] >= 0 && (cnt[c] == 0 || lists[c] != nullptr), "observation list missing");
        std::vector<std::array<int, 3>> v;
        for (int r = 0; r < cnt[c]; ++r) {
            EMS_CHECK_ARG(f->in_e(c, lists[c] + 3 * r), "observation index outside the field array");
            v.push_back({lists[c][3 * r], lists[c][3 * r + 1], lists[c][3 * r + 2]});
        }
        f->obs_lists.push_back(v);
        f->obs_n.push_back(cnt[c]);
    }
}

void fdtd_set_material(Sim *s, const double *eps, const double *sigma) { static_cast<FdtdSim *>(s)->set_material(eps, sigma); }

}  // namespace ems
