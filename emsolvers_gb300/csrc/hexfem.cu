// Hexahedral edge-element FEM (orders 1-3) of the fem_v2 family on one GPU:
// leapfrog (fem_v2/fem_simulation.cpp:560-655), 2nd-order symplectic
// (symplectic_2/fem_simulation.cpp:557-672) and its 4th-order triple jump
// (symplectic_4/fem_simulation.cpp:1280-1281,1347-1350).
//
// The reference applies the dense element matrix per element and scatters
// with atomics (fem_v2/fem_kernels.hpp:13-175).  Here every edge DOF gathers
// the contributions of the (at most four) elements that contain it, so there
// are no atomics and results are deterministic.  In FP64 the contributions
// are summed in the reference's element-visiting order (outer elements of
// fem_simulation.cpp:424-455 first, then inner elements) with unfused
// operations, and the source enters between the outer and inner sweeps as in
// the reference; the result is bit-identical to the serial reference.
#include <cuda_runtime.h>

#include <cmath>
#include <fstream>
#include <iomanip>

#include "ems_internal.hpp"

namespace ems {

__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }

constexpr int kMaxSrc = 8;

struct HexGeom {
    int o, gx, gy, gz, EX, EY, EZ, nouter, dof, total;
    size_t nc[3];
};

// Rank of element (i,j,k) in the reference's visiting order.
__device__ __forceinline__ int elem_rank(const HexGeom &g, int i, int j, int k)
{
    const int EX = g.EX, EY = g.EY, EZ = g.EZ;
    if (k == 0) return i + j * EX;
    if (k == EZ - 1) return EX * EY + i + j * EX;
    int b = 2 * EX * EY;
    if (i == 0) return b + j + (k - 1) * EY;
    if (i == EX - 1) return b + EY * (EZ - 2) + j + (k - 1) * EY;
    b += 2 * EY * (EZ - 2);
    if (j == 0) return b + (k - 1) + (i - 1) * (EZ - 2);
    if (j == EY - 1) return b + (EZ - 2) * (EX - 2) + (k - 1) + (i - 1) * (EZ - 2);
    return g.nouter + (i - 1) + (j - 1) * (EX - 2) + (k - 1) * (EX - 2) * (EY - 2);
}

__device__ __forceinline__ bool on_pec(const HexGeom &g, int c, int ix, int iy, int iz)
{
    if (c == 0) return iy == 0 || iy == g.gy || iz == 0 || iz == g.gz;
    if (c == 1) return ix == 0 || ix == g.gx || iz == 0 || iz == g.gz;
    return ix == 0 || ix == g.gx || iy == 0 || iy == g.gy;
}

struct SrcList {
    int n;
    int comp[kMaxSrc];
    int idx[kMaxSrc];
    double val[kMaxSrc];
};

// Force on one DOF: sum over the containing elements of row r of K times the
// element's gathered local vector.  sign -1: fem_v2 (-=), +1: symplectic (+=).
// EXACT: reference order and unfused FP ops; otherwise FMA accumulation.
template <class T, int O, bool EXACT>
__device__ T dof_force(const HexGeom &g, const T *__restrict__ K, const T *const lv[3], int c, int ix, int iy, int iz,
                       T sign, bool has_src, T srcval)
{
    constexpr int D = O * (O + 1) * (O + 1);
    constexpr int TT = 3 * D;
    // candidate element coordinates and local offsets per axis
    int ec[3][2], lc[3][2], nc_[3];
    const int pos[3] = {ix, iy, iz};
    const int ne[3] = {g.EX, g.EY, g.EZ};
    for (int d = 0; d < 3; ++d) {
        int p = pos[d];
        int e0 = p / O;
        nc_[d] = 0;
        if (d == c) {  // along the edge direction: exactly one element
            if (e0 < ne[d]) { ec[d][0] = e0; lc[d][0] = p - O * e0; nc_[d] = 1; }
        } else {
            if (e0 < ne[d]) { ec[d][nc_[d]] = e0; lc[d][nc_[d]] = p - O * e0; ++nc_[d]; }
            if (p % O == 0 && e0 - 1 >= 0 && e0 - 1 < ne[d]) { ec[d][nc_[d]] = e0 - 1; lc[d][nc_[d]] = O; ++nc_[d]; }
        }
    }
    int cnt = 0, rk[4], ex_[4], ey_[4], ez_[4], row[4];
    for (int a = 0; a < nc_[0]; ++a)
        for (int b = 0; b < nc_[1]; ++b)
            for (int q = 0; q < nc_[2]; ++q) {
                int l = lc[0][a], m = lc[1][b], n = lc[2][q], r;
                if (c == 0) r = l + m * O + n * O * (O + 1);
                else if (c == 1) r = D + l + m * (O + 1) + n * O * (O + 1);
                else r = 2 * D + l + m * (O + 1) + n * (O + 1) * (O + 1);
                ex_[cnt] = ec[0][a]; ey_[cnt] = ec[1][b]; ez_[cnt] = ec[2][q]; row[cnt] = r;
                rk[cnt] = EXACT ? elem_rank(g, ec[0][a], ec[1][b], ec[2][q]) : cnt;
                ++cnt;
            }
    if (EXACT)  // insertion sort by visiting rank
        for (int a = 1; a < cnt; ++a)
            for (int b = a; b > 0 && rk[b - 1] > rk[b]; --b) {
                int t;
                t = rk[b]; rk[b] = rk[b - 1]; rk[b - 1] = t;
                t = ex_[b]; ex_[b] = ex_[b - 1]; ex_[b - 1] = t;
                t = ey_[b]; ey_[b] = ey_[b - 1]; ey_[b - 1] = t;
                t = ez_[b]; ez_[b] = ez_[b - 1]; ez_[b - 1] = t;
                t = row[b]; row[b] = row[b - 1]; row[b - 1] = t;
            }
    T acc = 0;
    bool src_done = !has_src;
    const int gx = g.gx, gy = g.gy;
    for (int e = 0; e < cnt; ++e) {
        if (!src_done && rk[e] >= g.nouter) { acc = xadd(acc, srcval); src_done = true; }
        const T *Kr = K + (size_t)row[e] * TT;
        const int fx = O * ex_[e], fy = O * ey_[e], fz = O * ez_[e];
        T temp = 0;
        int mm = 0;
        for (int n = 0; n < O + 1; ++n)
            for (int m = 0; m < O + 1; ++m)
                for (int l = 0; l < O; ++l, ++mm) {
                    T v = lv[0][(size_t)(fx + l) + (size_t)(fy + m) * gx + (size_t)(fz + n) * gx * (gy + 1)];
                    temp = EXACT ? xadd(temp, xmul(Kr[mm], v)) : fma(Kr[mm], v, temp);
                }
        for (int n = 0; n < O + 1; ++n)
            for (int m = 0; m < O; ++m)
                for (int l = 0; l < O + 1; ++l, ++mm) {
                    T v = lv[1][(size_t)(fx + l) + (size_t)(fy + m) * (gx + 1) + (size_t)(fz + n) * (gx + 1) * gy];
                    temp = EXACT ? xadd(temp, xmul(Kr[mm], v)) : fma(Kr[mm], v, temp);
                }
        for (int n = 0; n < O; ++n)
            for (int m = 0; m < O + 1; ++m)
                for (int l = 0; l < O + 1; ++l, ++mm) {
                    T v = lv[2][(size_t)(fx + l) + (size_t)(fy + m) * (gx + 1) + (size_t)(fz + n) * (gx + 1) * (gy + 1)];
                    temp = EXACT ? xadd(temp, xmul(Kr[mm], v)) : fma(Kr[mm], v, temp);
                }
        acc = sign < 0 ? xsub(acc, temp) : xadd(acc, temp);
    }
    if (!src_done) acc = xadd(acc, srcval);
    return acc;
}

__device__ __forceinline__ void dof_coords(const HexGeom &g, int c, size_t t, int &ix, int &iy, int &iz)
{
    int nxc = c == 0 ? g.gx : g.gx + 1;
    int nyc = c == 1 ? g.gy : g.gy + 1;
    ix = (int)(t % nxc);
    size_t r = t / nxc;
    iy = (int)(r % nyc);
    iz = (int)(r / nyc);
}

// Leapfrog step, one thread per DOF: E2 = (-K E1, boundary zeroed) + 2 E1 - E0,
// then the point source, then PEC (fem_v2/fem_simulation.cpp:576-654, 1115).
template <class T, int O, bool EXACT>
__global__ void __launch_bounds__(128) hex_leapfrog_kernel(HexGeom g, const T *__restrict__ K, const T *E1x, const T *E1y,
                                                           const T *E1z, const T *E0x, const T *E0y, const T *E0z,
                                                           T *E2x, T *E2y, T *E2z, SrcList src)
{
    const int c = blockIdx.y;
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nc[c]) return;
    int ix, iy, iz;
    dof_coords(g, c, t, ix, iy, iz);
    const T *lv[3] = {E1x, E1y, E1z};
    T f = 0;
    bool pec = on_pec(g, c, ix, iy, iz);
    if (!pec) f = dof_force<T, O, EXACT>(g, K, lv, c, ix, iy, iz, T(-1), false, T(0));
    const T *e1 = c == 0 ? E1x : c == 1 ? E1y : E1z;
    const T *e0 = c == 0 ? E0x : c == 1 ? E0y : E0z;
    T v = xadd(f, xsub(xmul(T(2), e1[t]), e0[t]));
    for (int s = 0; s < src.n; ++s)
        if (src.comp[s] == c && (size_t)src.idx[s] == t) v = xsub(v, (T)src.val[s]);
    if (pec) v = 0;
    T *e2 = c == 0 ? E2x : c == 1 ? E2y : E2z;
    e2[t] = v;
}

// Symplectic kick: F = K U (+ source between outer and inner elements),
// boundary F zeroed, P -= dt F (symplectic_2/fem_simulation.cpp:603-653).
// F is also stored (the reference keeps it in level 2).
template <class T, int O, bool EXACT>
__global__ void __launch_bounds__(128) hex_kick_kernel(HexGeom g, const T *__restrict__ K, const T *Ux, const T *Uy, const T *Uz,
                                                       T *Px, T *Py, T *Pz, T *Fx, T *Fy, T *Fz, T dt, SrcList src)
{
    const int c = blockIdx.y;
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nc[c]) return;
    int ix, iy, iz;
    dof_coords(g, c, t, ix, iy, iz);
    const T *lv[3] = {Ux, Uy, Uz};
    bool has = false;
    T sv = 0;
    for (int s = 0; s < src.n; ++s)
        if (src.comp[s] == c && (size_t)src.idx[s] == t) { has = true; sv = (T)src.val[s]; }
    T f = 0;
    if (!on_pec(g, c, ix, iy, iz)) f = dof_force<T, O, EXACT>(g, K, lv, c, ix, iy, iz, T(1), has, sv);
    T *F = c == 0 ? Fx : c == 1 ? Fy : Fz;
    T *P = c == 0 ? Px : c == 1 ? Py : Pz;
    F[t] = f;
    P[t] = EXACT ? xsub(P[t], xmul(dt, f)) : fma(-dt, f, P[t]);
}

// Drift U += coef * P / m (symplectic_2/fem_simulation.cpp:583-601, 647-668);
// coef = 0.5*deltat, inv_m = 8/o^3 as in the reference's operand order; with
// `pec` set, U and P are zeroed on the boundary afterwards (1132-1276).
template <class T, bool EXACT>
__global__ void hex_drift_kernel(HexGeom g, T *Ux, T *Uy, T *Uz, T *Px, T *Py, T *Pz, T coef, T m, int pec)
{
    const int c = blockIdx.y;
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nc[c]) return;
    T *U = c == 0 ? Ux : c == 1 ? Uy : Uz;
    T *P = c == 0 ? Px : c == 1 ? Py : Pz;
    T u = EXACT ? xadd(U[t], (T)(xmul(coef, P[t]) / m)) : U[t] + coef * P[t] / m;
    if (pec) {
        int ix, iy, iz;
        dof_coords(g, c, t, ix, iy, iz);
        if (on_pec(g, c, ix, iy, iz)) { u = 0; P[t] = 0; }
    }
    U[t] = u;
}

// Receivers: fem_v2/fem_simulation.cpp:1273-1312 (one thread per receiver).
template <class T>
__global__ void hex_sample_kernel(HexGeom g, const T *Lx, const T *Ly, const T *Lz, int nobs, const int *obs, double *tr, int nsamp, int s)
{
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nobs) return;
    const int gx = g.gx, gy = g.gy;
    int ox = obs[3 * o], oy = obs[3 * o + 1], oz = obs[3 * o + 2];
    double *out = tr + ((size_t)o * nsamp + s) * 4;
    double a = __dadd_rn(__dadd_rn(__dadd_rn((double)Lx[ox - 1], (double)Lx[ox]), (double)Lx[ox + gx * (gy + 1) - 1]), (double)Lx[ox + gx * (gy + 1)]);
    double b = __dadd_rn(__dadd_rn(__dadd_rn((double)Ly[oy - (gx + 1)], (double)Ly[oy]), (double)Ly[oy + (gx + 1) * (gy - 1)]), (double)Ly[oy + (gx + 1) * gy]);
    out[1] = a / 4.0;
    out[2] = b / 4.0;
    out[3] = (double)Lz[oz];
}

static double femv2_source(double t)
{
    const double freq = 1.0e9;
    const double chi = 1.0 / freq;
    double delay = t - chi;
    double zeta = 2.0 * M_PI * M_PI * freq * freq;
    return 2.0 * zeta * (2.0 * zeta * delay * delay - 1.0) * std::exp(0.0 - zeta * delay * delay) * 0.001;
}

struct HexFemSim : Sim {
    ems_hexfem_params P;
    std::string kdir;
    HexGeom g{};
    bool fp64, exact;
    DevBuf lev[3];         // per component: 3 levels
    DevBuf dK;
    std::vector<double> Kh;
    std::vector<std::array<int, 4>> srcs;   // comp, flat index
    std::vector<std::array<int, 3>> obs_idx; // x, y, z flat indices
    std::vector<std::array<int, 3>> obs_ijk;
    int l0 = 0, l1 = 1, l2 = 2;              // leapfrog ring
    double cur_time = 0.0;
    DevBuf d_obs, d_tr;

    explicit HexFemSim(const ems_hexfem_params *p) : Sim(Kind::HEXFEM), P(*p)
    {
        kdir = P.kmat_dir ? P.kmat_dir : "kmat";
        P.kmat_dir = nullptr;
        EMS_CHECK_ARG(P.order >= 1 && P.order <= 3, "order must be 1, 2 or 3");
        EMS_CHECK_ARG(P.integrator == EMS_LEAPFROG || P.integrator == EMS_SYMP2 || P.integrator == EMS_SYMP4,
                      "hexahedral integrator must be EMS_LEAPFROG, EMS_SYMP2 or EMS_SYMP4");
        EMS_CHECK_ARG(P.precision == EMS_FP64 || P.precision == EMS_FP32, "precision must be EMS_FP64 or EMS_FP32");
        EMS_CHECK_ARG(P.h > 0 && P.dt > 0 && P.permittivity > 0 && P.permeability > 0, "h, dt, eps, mu must be positive");
        EMS_CHECK_ARG(P.time_frequency > 0, "time_frequency must be positive");
        int o = P.order;
        g.o = o; g.gx = P.grid[0]; g.gy = P.grid[1]; g.gz = P.grid[2];
        g.EX = g.gx / o; g.EY = g.gy / o; g.EZ = g.gz / o;
        // with fewer than two elements per direction the reference's outer
        // list visits boundary elements twice; such grids are rejected
        EMS_CHECK_ARG(g.EX >= 2 && g.EY >= 2 && g.EZ >= 2, "need at least two elements per direction");
        double c = 1.0 / std::sqrt(P.permittivity * P.permeability);
        EMS_CHECK_ARG(c * P.dt < P.h, "time step violates c*dt < h (reference check_params)");
        g.dof = o * (o + 1) * (o + 1);
        g.total = 3 * g.dof;
        g.nouter = 2 * g.EX * g.EY + 2 * g.EY * (g.EZ - 2) + 2 * (g.EZ - 2) * (g.EX - 2);
        g.nc[0] = (size_t)g.gx * (g.gy + 1) * (g.gz + 1);
        g.nc[1] = (size_t)(g.gx + 1) * g.gy * (g.gz + 1);
        g.nc[2] = (size_t)(g.gx + 1) * (g.gy + 1) * g.gz;
        fp64 = P.precision == EMS_FP64;
        exact = fp64;
        // element matrix (fem_v2/fem_simulation.cpp:458-490, symplectic_2 473)
        std::string fn = kdir + "/" + (P.use_ofem ? std::to_string(o) : "lamped" + std::to_string(o)) + ".csv";
        auto M = load_matrix_csv(fn);
        int T = g.total;
        if ((int)M.size() != T) throw Error{EMS_ERR_IO, fn + ": expected " + std::to_string(T) + " rows"};
        for (auto &r : M)
            if ((int)r.size() != T) throw Error{EMS_ERR_IO, fn + ": expected " + std::to_string(T) + " columns"};
        double scale;
        if (P.integrator == EMS_LEAPFROG)
            scale = 4.0 * P.dt * P.dt / (P.h * o) / (P.h * o) / P.permeability / P.permittivity / (8.0 / o / o / o);
        else
            scale = 4.0 / (P.h * o) / (P.h * o) / P.permeability / P.permittivity;
        Kh.resize((size_t)T * T);
        for (int i = 0; i < T; ++i)
            for (int j = 0; j < T; ++j) Kh[(size_t)i * T + j] = scale * M[i][j];
        init_stream();
        size_t w = fp64 ? 8 : 4;
        for (int q = 0; q < 3; ++q) { lev[q].alloc(3 * g.nc[q] * w); lev[q].zero(stream); }
        if (fp64) {
            dK.alloc(Kh.size() * 8);
            EMS_CUDA(cudaMemcpyAsync(dK.p, Kh.data(), Kh.size() * 8, cudaMemcpyHostToDevice, stream));
        } else {
            std::vector<float> kf(Kh.begin(), Kh.end());
            dK.alloc(kf.size() * 4);
            EMS_CUDA(cudaMemcpyAsync(dK.p, kf.data(), kf.size() * 4, cudaMemcpyHostToDevice, stream));
        }
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    int flat(int c, const int *q) const
    {
        if (c == 0) return q[0] + q[1] * g.gx + q[2] * g.gx * (g.gy + 1);
        if (c == 1) return q[0] + q[1] * (g.gx + 1) + q[2] * (g.gx + 1) * g.gy;
        return q[0] + q[1] * (g.gx + 1) + q[2] * (g.gx + 1) * (g.gy + 1);
    }

    template <class T> T *L(int c, int level) const { return lev[c].as<T>() + (size_t)level * g.nc[c]; }

    template <class T, int O> void launch_leapfrog(const SrcList &s)
    {
        size_t mx = std::max(g.nc[0], std::max(g.nc[1], g.nc[2]));
        dim3 grid((unsigned)((mx + 127) / 128), 3);
        auto k = exact ? hex_leapfrog_kernel<T, O, true> : hex_leapfrog_kernel<T, O, false>;
        k<<<grid, 128, 0, stream>>>(g, dK.as<T>(), L<T>(0, l1), L<T>(1, l1), L<T>(2, l1), L<T>(0, l0), L<T>(1, l0), L<T>(2, l0),
                                    L<T>(0, l2), L<T>(1, l2), L<T>(2, l2), s);
    }
    template <class T, int O> void launch_kick(T dt, const SrcList &s)
    {
        size_t mx = std::max(g.nc[0], std::max(g.nc[1], g.nc[2]));
        dim3 grid((unsigned)((mx + 127) / 128), 3);
        auto k = exact ? hex_kick_kernel<T, O, true> : hex_kick_kernel<T, O, false>;
        k<<<grid, 128, 0, stream>>>(g, dK.as<T>(), L<T>(0, 0), L<T>(1, 0), L<T>(2, 0), L<T>(0, 1), L<T>(1, 1), L<T>(2, 1),
                                    L<T>(0, 2), L<T>(1, 2), L<T>(2, 2), dt, s);
    }
    template <class T> void launch_drift(T coef, int pec)
    {
        size_t mx = std::max(g.nc[0], std::max(g.nc[1], g.nc[2]));
        dim3 grid((unsigned)((mx + 255) / 256), 3);
        T m = (T)(8.0 / g.o / g.o / g.o);
        auto k = exact ? hex_drift_kernel<T, true> : hex_drift_kernel<T, false>;
        k<<<grid, 256, 0, stream>>>(g, L<T>(0, 0), L<T>(1, 0), L<T>(2, 0), L<T>(0, 1), L<T>(1, 1), L<T>(2, 1), coef, m, pec);
    }

    SrcList sources(double val) const
    {
        SrcList s{};
        s.n = (int)srcs.size();
        for (int q = 0; q < s.n; ++q) { s.comp[q] = srcs[q][0]; s.idx[q] = srcs[q][1]; s.val[q] = val; }
        return s;
    }

    template <class T, int O> void run_o(int nsteps)
    {
        const int tf = P.time_frequency;
        nobs = (int)obs_idx.size();
        nsamp = nsteps > 0 ? (nsteps - 1) / tf + 1 : 0;
        ncols = 4;
        std::vector<int> oi;
        for (auto &q : obs_idx) { oi.push_back(q[0]); oi.push_back(q[1]); oi.push_back(q[2]); }
        if (oi.empty()) oi.assign(3, 0);
        d_obs.alloc(oi.size() * 4);
        EMS_CUDA(cudaMemcpyAsync(d_obs.p, oi.data(), oi.size() * 4, cudaMemcpyHostToDevice, stream));
        size_t ntr = (size_t)std::max(nobs, 1) * std::max(nsamp, 1) * 4;
        d_tr.alloc(ntr * 8);
        d_tr.zero(stream);
        std::vector<double> times(std::max(nsamp, 1), 0.0);
        long long launches = 0;
        const double x1 = 1.0 / (2.0 - std::pow(2.0, 1.0 / 3.0)), x2 = 1.0 - 2.0 * x1;
        const int o = g.o;
        EMS_CUDA(cudaEventRecord(ev0, stream));
        for (int step = 0; step < nsteps; ++step) {
            bool samp = nobs > 0 && step % tf == 0;
            if (P.integrator == EMS_LEAPFROG) {
                // fem_v2 samples level 1 (E^n) after computing E^{n+1}; E^n is untouched by the step
                if (samp) {
                    hex_sample_kernel<T><<<(nobs + 63) / 64, 64, 0, stream>>>(g, L<T>(0, l1), L<T>(1, l1), L<T>(2, l1), nobs, d_obs.as<int>(), d_tr.as<double>(), nsamp, step / tf);
                    times[step / tf] = cur_time;
                    ++launches;
                }
                double sv = femv2_source(cur_time) * P.dt * P.dt / P.permittivity / P.h / P.h / P.h;
                launch_leapfrog<T, O>(sources(sv));
                ++launches;
                l0 = (l0 + 1) % 3; l1 = (l1 + 1) % 3; l2 = (l2 + 1) % 3;
            } else {
                if (samp) {
                    hex_sample_kernel<T><<<(nobs + 63) / 64, 64, 0, stream>>>(g, L<T>(0, 0), L<T>(1, 0), L<T>(2, 0), nobs, d_obs.as<int>(), d_tr.as<double>(), nsamp, step / tf);
                    times[step / tf] = cur_time;
                    ++launches;
                }
                double sub[3], off[3];
                int nsub;
                if (P.integrator == EMS_SYMP2) { nsub = 1; sub[0] = P.dt; off[0] = 0.0; }
                else { nsub = 3; sub[0] = x1 * P.dt; off[0] = 0.0; sub[1] = x2 * P.dt; off[1] = x1 * P.dt; sub[2] = x1 * P.dt; off[2] = (x1 + x2) * P.dt; }
                for (int q = 0; q < nsub; ++q) {
                    double deltat = sub[q];
                    double sv = femv2_source(cur_time + off[q] + 0.5 * deltat) * 8.0 / P.permittivity / (P.h * o) / (P.h * o) / (P.h * o);
                    if (exact || q == 0) launch_drift<T>((T)(0.5 * deltat), 0), ++launches;
                    launch_kick<T, O>((T)deltat, sources(sv));
                    ++launches;
                    if (exact || q == nsub - 1) launch_drift<T>((T)(0.5 * deltat), 1);
                    else launch_drift<T>((T)(0.5 * deltat + 0.5 * sub[q + 1]), 1);
                    ++launches;
                }
            }
            cur_time += P.dt;
        }
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaEventRecord(ev1, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        float ms = 0;
        EMS_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        last_ms = ms;
        last_launches = launches;
        traces.assign(ntr, 0.0);
        EMS_CUDA(cudaMemcpy(traces.data(), d_tr.p, ntr * 8, cudaMemcpyDeviceToHost));
        traces.resize((size_t)nobs * nsamp * 4);
        for (int ob = 0; ob < nobs; ++ob)
            for (int s = 0; s < nsamp; ++s) traces[((size_t)ob * nsamp + s) * 4] = times[s];
    }

    template <class T> void run_t(int nsteps)
    {
        if (g.o == 1) run_o<T, 1>(nsteps);
        else if (g.o == 2) run_o<T, 2>(nsteps);
        else run_o<T, 3>(nsteps);
    }

    void run(int nsteps) override
    {
        EMS_CHECK_ARG(nsteps >= 0, "num_steps must be >= 0");
        EMS_CHECK_ARG(srcs.size() <= (size_t)kMaxSrc, "at most 8 point sources");
        if (fp64) run_t<double>(nsteps); else run_t<float>(nsteps);
        const size_t w = fp64 ? 8 : 4;
        check_finite({{lev[0].p, lev[0].bytes / w}, {lev[1].p, lev[1].bytes / w}, {lev[2].p, lev[2].bytes / w}}, fp64);
    }

    size_t field_size(int which) const override
    {
        if (which < 0 || which > 2) throw Error{EMS_ERR_INVALID_ARGUMENT, "field index must be 0..2 (x, y, z components)"};
        return 3 * g.nc[which];
    }
    // levels returned in the reference's storage order (ring index 0,1,2)
    void get_field(int which, double *out) const override
    {
        size_t cnt = field_size(which);
        if (fp64) {
            EMS_CUDA(cudaMemcpy(out, lev[which].p, cnt * 8, cudaMemcpyDeviceToHost));
        } else {
            std::vector<float> tmp(cnt);
            EMS_CUDA(cudaMemcpy(tmp.data(), lev[which].p, cnt * 4, cudaMemcpyDeviceToHost));
            for (size_t q = 0; q < cnt; ++q) out[q] = tmp[q];
        }
    }
    void set_field(int which, const double *in) override
    {
        size_t cnt = field_size(which);
        if (fp64) {
            EMS_CUDA(cudaMemcpy(lev[which].p, in, cnt * 8, cudaMemcpyHostToDevice));
        } else {
            std::vector<float> tmp(in, in + cnt);
            EMS_CUDA(cudaMemcpy(lev[which].p, tmp.data(), cnt * 4, cudaMemcpyHostToDevice));
        }
    }

    // fem_v2/fem_simulation.cpp:1322-1344: setprecision(15) scientific,
    // header time,Ex,Ey,Ez.  The reference writes every receiver to the same
    // name; here receiver i > 0 gets the suffix _<i> before the extension.
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
            f << std::setprecision(15) << std::scientific;
            f << "time,Ex,Ey,Ez" << std::endl;
            for (int s = 0; s < nsamp; ++s) {
                const double *r = &traces[((size_t)o * nsamp + s) * 4];
                f << r[0] << "," << r[1] << "," << r[2] << "," << r[3] << std::endl;
            }
        }
    }

    void reset() override
    {
        for (int q = 0; q < 3; ++q) lev[q].zero(stream);
        l0 = 0; l1 = 1; l2 = 2;
        cur_time = 0.0;
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    void time_dominant(int launches, double *ms, double *bytes, std::string *name) override
    {
        size_t w = fp64 ? 8 : 4;
        size_t ndof = g.nc[0] + g.nc[1] + g.nc[2];
        std::vector<DevBuf> save(3);
        for (int q = 0; q < 3; ++q) {
            save[q].alloc(lev[q].bytes);
            EMS_CUDA(cudaMemcpyAsync(save[q].p, lev[q].p, lev[q].bytes, cudaMemcpyDeviceToDevice, stream));
        }
        auto body = [&](auto tag) {
            using T = decltype(tag);
            SrcList s = sources(0.0);
            for (int r = 0; r <= launches; ++r) {
                if (r == 1) EMS_CUDA(cudaEventRecord(ev0, stream));
                auto go = [&](auto oc) {
                    constexpr int O = decltype(oc)::value;
                    if (P.integrator == EMS_LEAPFROG) launch_leapfrog<T, O>(s); else launch_kick<T, O>((T)P.dt, s);
                };
                if (g.o == 1) go(std::integral_constant<int, 1>());
                else if (g.o == 2) go(std::integral_constant<int, 2>());
                else go(std::integral_constant<int, 3>());
            }
        };
        if (fp64) body(double()); else body(float());
        EMS_CUDA(cudaEventRecord(ev1, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        float t = 0;
        EMS_CUDA(cudaEventElapsedTime(&t, ev0, ev1));
        for (int q = 0; q < 3; ++q)
            EMS_CUDA(cudaMemcpyAsync(lev[q].p, save[q].p, lev[q].bytes, cudaMemcpyDeviceToDevice, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        *ms = t / launches;
        // leapfrog: read E^n, E^{n-1}, write E^{n+1}; kick: read U, read/write P, write F
        *bytes = (double)ndof * w * (P.integrator == EMS_LEAPFROG ? 3.0 : 4.0);
        *name = std::string(P.integrator == EMS_LEAPFROG ? "hex_leapfrog_kernel" : "hex_kick_kernel") + "<o=" + std::to_string(g.o) + ">";
    }
};

Sim *make_hexfem(const ems_hexfem_params *p) { return new HexFemSim(p); }

void hexfem_set_source(Sim *s, int comp, const int ijk[3])
{
    auto *f = static_cast<HexFemSim *>(s);
    EMS_CHECK_ARG(comp >= 0 && comp < 3 && ijk, "component must be 0, 1 or 2");
    int lim[3] = {f->g.gx - (comp == 0), f->g.gy - (comp == 1), f->g.gz - (comp == 2)};
    for (int d = 0; d < 3; ++d) EMS_CHECK_ARG(ijk[d] >= 0 && ijk[d] <= lim[d], "source edge outside the grid");
    EMS_CHECK_ARG(f->srcs.size() < (size_t)kMaxSrc, "at most 8 point sources");
    f->srcs.push_back({comp, f->flat(comp, ijk), 0, 0});
}

void hexfem_add_observation(Sim *s, const int ijk[3])
{
    auto *f = static_cast<HexFemSim *>(s);
    EMS_CHECK_ARG(ijk != nullptr, "position required");
    // the sample reads x-edges (i-1..i, j, k..k+1), y-edges (i, j-1..j, k..k+1), z-edge (i,j,k)
    EMS_CHECK_ARG(ijk[0] >= 1 && ijk[0] < f->g.gx && ijk[1] >= 1 && ijk[1] < f->g.gy && ijk[2] >= 0 && ijk[2] < f->g.gz,
                  "observation point must be an interior node");
    f->obs_idx.push_back({f->flat(0, ijk), f->flat(1, ijk), f->flat(2, ijk)});
    f->obs_ijk.push_back({ijk[0], ijk[1], ijk[2]});
}

}  // namespace ems
