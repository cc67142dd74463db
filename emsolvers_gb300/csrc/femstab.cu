// Stabilised order-1 hexahedral edge-element solver (the reference's fem/
// directory) on one GPU.
//
// E lives on the primal edges (fem/fem_simulation.cpp:61-123, cyclic local
// order); a step is the three-level update E^{n+1} = -K E^n + 2 E^n - E^{n-1}
// (466-634) with the element matrix K = dt^2 / (2 mu eps h^2) Ct Bt^-1 At,
// At = A + s Abar, Bt = B + s Bbar, Ct = C + s Cbar (125-434), in the
// conventional or the orthogonal (OFEM) basis, then point sources, the
// x-directed Hertz dipole (636-740) and PEC (743-833).  The reference scatters
// element rows with atomics; here every edge DOF gathers them from the (at
// most four) elements that contain it in the reference's element order, so
// the FP64 result is bit-identical to the serial reference.
//
// The element matrices are built from their structure (see build_parts):
// A holds, on the four rows of a component, one half of the element-averaged
// discrete curl of that component; B is the tensor-product edge mass of each
// component; C = Bbar = A^T and Cbar = Abar^T; Abar is the stabilisation,
// which in the modal basis of each component (constant, linear along either
// transverse axis, bilinear) couples every non-constant mode with the
// matching modes of the other components.  The OFEM basis is that modal
// basis.  Every entry is an integer or a correctly rounded k/3 or k/9.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <fstream>

#include "ems_internal.hpp"
#include "hexedge.cuh"

namespace ems {

namespace {

// One update gathered per edge DOF: E2_r = -(sum over the elements e that
// contain edge r, in increasing element index, of (K E1_e)_l) + (2 E1 - E0),
// zero on PEC edges.  EXACT (FP64): explicitly rounded operations in the
// reference's order (temp = sum_m K_lm e_m, E2 -= temp element by element);
// FP32: fused multiply-adds.
template <class T, bool EXACT>
__global__ void __launch_bounds__(128) femstab_sweep_kernel(HexGeom g, const T *__restrict__ K, const T *__restrict__ E0,
                                                            const T *__restrict__ E1, T *__restrict__ E2)
{
    const int c = blockIdx.y;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n[c]) return;
    const size_t off[3] = {0, g.n[0], g.n[0] + g.n[1]};
    int i, j, k;
    hex_coords(g, c, t, i, j, k);
    // the elements holding the edge as local edge q, in increasing element
    // index (offsets on the two transverse axes of the cyclic order)
    const int ord[3][4] = {{3, 2, 1, 0}, {3, 1, 2, 0}, {3, 2, 1, 0}};
    T acc = 0;
    for (int oi = 0; oi < 4; ++oi) {
        const int q = ord[c][oi], a0 = q & 1, a1 = q >> 1;
        int ci = i, cj = j, ck = k;
        if (c == 0) { cj -= a0; ck -= a1; }
        else if (c == 1) { ck -= a0; ci -= a1; }
        else { ci -= a0; cj -= a1; }
        if (ci < 0 || cj < 0 || ck < 0 || ci >= g.gx || cj >= g.gy || ck >= g.gz) continue;
        const T *Kr = K + (4 * c + q) * 12;
        T temp = 0;
#pragma unroll
        for (int m = 0; m < 12; ++m) {
            const T e = E1[off[m >> 2] + hex_edge(g, m >> 2, ci, cj, ck, m & 3)];
            temp = EXACT ? ad(temp, ml(Kr[m], e)) : fma(Kr[m], e, temp);
        }
        acc = EXACT ? sb(acc, temp) : acc - temp;
    }
    const T e1 = E1[off[c] + t], e0 = E0[off[c] + t];
    T e2 = EXACT ? ad(acc, sb(ml(T(2), e1), e0)) : acc + (T(2) * e1 - e0);
    if (hex_e_pec(g, c, i, j, k)) e2 = 0;
    E2[off[c] + t] = e2;
}

// fem/fem_simulation.cpp:28-38: f0 = 1 GHz, times mu / h^3 and dl = 1 mm
double femstab_source(double t, double mu, double h)
{
    const double f0 = 1.0e9;
    return 4.0 * M_PI * M_PI * f0 * f0 * (1.0 - 4.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) * (t - 1.0 / f0)) *
           std::exp(-2.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) * (t - 1.0 / f0)) * mu / h / h / h * 0.001;
}

using Mat12 = std::array<double, 144>;

Mat12 mat_mul(const Mat12 &a, const Mat12 &b)
{
    Mat12 c{};
    for (int i = 0; i < 12; ++i)
        for (int j = 0; j < 12; ++j) {
            double s = 0.0;
            for (int k = 0; k < 12; ++k) s += a[i * 12 + k] * b[k * 12 + j];
            c[i * 12 + j] = s;
        }
    return c;
}

Mat12 transposed(const Mat12 &a)
{
    Mat12 b{};
    for (int i = 0; i < 12; ++i)
        for (int j = 0; j < 12; ++j) b[j * 12 + i] = a[i * 12 + j];
    return b;
}

// Inverse by Gauss-Jordan elimination with partial pivoting (the first row
// of largest magnitude), the pivot row scaled, then eliminated from every
// other row.
Mat12 gauss_jordan_inverse(Mat12 a)
{
    Mat12 inv{};
    for (int i = 0; i < 12; ++i) inv[i * 12 + i] = 1.0;
    for (int col = 0; col < 12; ++col) {
        int piv = col;
        for (int i = col + 1; i < 12; ++i)
            if (std::fabs(a[i * 12 + col]) > std::fabs(a[piv * 12 + col])) piv = i;
        if (a[piv * 12 + col] == 0.0) throw Error{EMS_ERR_INVALID_ARGUMENT, "element mass matrix is singular"};
        if (piv != col)
            for (int j = 0; j < 12; ++j) {
                std::swap(a[piv * 12 + j], a[col * 12 + j]);
                std::swap(inv[piv * 12 + j], inv[col * 12 + j]);
            }
        const double d = a[col * 12 + col];
        for (int j = 0; j < 12; ++j) { a[col * 12 + j] /= d; inv[col * 12 + j] /= d; }
        for (int i = 0; i < 12; ++i) {
            if (i == col) continue;
            const double f = a[i * 12 + col];
            if (f == 0.0) continue;
            for (int j = 0; j < 12; ++j) { a[i * 12 + j] -= f * a[col * 12 + j]; inv[i * 12 + j] -= f * inv[col * 12 + j]; }
        }
    }
    return inv;
}

// The six element matrices of one basis (fem/fem_simulation.cpp:125-409).
// T = diag(H, H, H) maps the four cyclic edges of a component to its modes
// (constant, sign by the first transverse offset, by the second, product);
// R couples each non-constant mode with the matching modes of the other
// components; the conventional Abar is T^T W R T / 16 with mode weights
// W = (0, 4, 4, 8/3), and the OFEM operators are A_o = T A, B_o = T B T^T,
// Bbar_o = T Bbar T^T, Abar_o = R T.  Integer arithmetic is exact in
// doubles; the divisions by 3 and 9 come last, so every entry is the
// correctly rounded value.
void build_parts(int use_ofem, Mat12 &A, Mat12 &Abar, Mat12 &B, Mat12 &Bbar, Mat12 &C, Mat12 &Cbar)
{
    static const double curl[3][12] = {{0, 0, 0, 0, 0.5, -0.5, 0.5, -0.5, -0.5, -0.5, 0.5, 0.5},
                                       {-0.5, -0.5, 0.5, 0.5, 0, 0, 0, 0, 0.5, -0.5, 0.5, -0.5},
                                       {0.5, -0.5, 0.5, -0.5, -0.5, -0.5, 0.5, 0.5, 0, 0, 0, 0}};
    static const double modes[4][4] = {{1, 1, 1, 1}, {-1, 1, -1, 1}, {-1, -1, 1, 1}, {1, -1, -1, 1}};
    static const int ax[3][2] = {{1, 2}, {2, 0}, {0, 1}};   // transverse axes in the cyclic order
    Mat12 T{}, R{}, Ac{}, B9{};
    for (int c = 0; c < 3; ++c)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) {
                T[(4 * c + a) * 12 + 4 * c + b] = modes[a][b];
                const int d = ((a ^ b) & 1) + ((a ^ b) >> 1);   // transverse axes on which a and b differ
                B9[(4 * c + a) * 12 + 4 * c + b] = (double)(8 >> d);
            }
    for (int c = 0; c < 3; ++c) {
        for (int m = 1; m <= 2; ++m) {
            const int t = ax[c][m - 1];
            R[(4 * c + m) * 12 + 4 * c + m] = 2.0;
            R[(4 * c + m) * 12 + 4 * t + (ax[t][0] == c ? 1 : 2)] = -2.0;
        }
        R[(4 * c + 3) * 12 + 4 * c + 3] = 2.0;
        for (int t = 0; t < 3; ++t)
            if (t != c) R[(4 * c + 3) * 12 + 4 * t + 3] = -1.0;
    }
    for (int r = 0; r < 144; ++r) Ac[r] = curl[r / 48][r % 12];
    const Mat12 Tt = transposed(T);
    if (!use_ofem) {
        A = Ac;
        static const double w3[4] = {0.0, 12.0, 12.0, 8.0};   // 3 W
        Mat12 x{};
        for (int r = 0; r < 144; ++r) x[r] = w3[(r / 12) % 4] * R[r];
        x = mat_mul(Tt, mat_mul(x, T));
        for (int r = 0; r < 144; ++r) Abar[r] = (x[r] / 16.0) / 3.0;
        for (int r = 0; r < 144; ++r) B[r] = B9[r] / 9.0;
        Bbar = transposed(Ac);
    } else {
        A = mat_mul(T, Ac);
        Abar = mat_mul(R, T);
        const Mat12 x = mat_mul(mat_mul(T, B9), Tt);
        for (int r = 0; r < 144; ++r) B[r] = x[r] / 9.0;
        Bbar = mat_mul(mat_mul(T, transposed(Ac)), Tt);
    }
    C = transposed(A);
    Cbar = transposed(Abar);
}

}  // namespace

// K = dt^2 / (2 mu eps h^2) Ct Bt^-1 At, formed in the reference's order
// (fem/fem_simulation.cpp:411): the scalar left to right, then
// ((s Ct) Bt^-1) At with plain row-column sums in index order.
std::array<double, 144> femstab_kmat(double dt, double mu, double eps, double h, double sf, int use_ofem)
{
    Mat12 A, Ab, B, Bb, C, Cb;
    build_parts(use_ofem, A, Ab, B, Bb, C, Cb);
    for (int r = 0; r < 144; ++r) {
        A[r] = A[r] + sf * Ab[r];
        B[r] = B[r] + sf * Bb[r];
        C[r] = C[r] + sf * Cb[r];
    }
    const Mat12 Bi = gauss_jordan_inverse(B);
    const double s0 = 0.5 * dt * dt / mu / eps / h / h;
    for (int r = 0; r < 144; ++r) C[r] = s0 * C[r];
    return mat_mul(mat_mul(C, Bi), A);
}

struct FemStabSim : Sim {
    ems_femstab_params P;
    HexGeom g{};
    bool fp64;
    size_t ntot;
    std::array<double, 144> K{};
    DevBuf dE, dK, d_src_idx, d_src_val, d_src_op, d_obs_cnt, d_obs_start, d_obs_idx, d_tr;
    std::vector<std::array<int, 4>> srcs;   // comp, i, j, k
    std::vector<std::array<int, 3>> dips;   // x-directed Hertz dipoles
    std::vector<std::vector<std::array<int, 3>>> obs_lists;
    std::vector<int> obs_n;
    int r0 = 0, r1 = 1, r2 = 2;             // storage slots of E^{n-1}, E^n, E^{n+1}
    double cur_time = 0.0;

    explicit FemStabSim(const ems_femstab_params *p) : Sim(Kind::HEXFEM), P(*p)
    {
        EMS_CHECK_ARG(P.precision == EMS_FP64 || P.precision == EMS_FP32, "precision must be EMS_FP64 or EMS_FP32");
        EMS_CHECK_ARG(P.h > 0 && P.dt > 0 && P.permittivity > 0 && P.permeability > 0, "h, dt, eps, mu must be positive");
        EMS_CHECK_ARG(P.time_frequency > 0, "time_frequency must be positive");
        EMS_CHECK_ARG(P.use_ofem == 0 || P.use_ofem == 1, "use_ofem must be 0 or 1");
        EMS_CHECK_ARG(std::isfinite(P.stabilization_factor), "stabilization_factor must be finite");
        EMS_CHECK_ARG(P.grid[0] >= 1 && P.grid[1] >= 1 && P.grid[2] >= 1, "grid sizes must be positive");
        // fem/fem_simulation.cpp:951-959 (check_params)
        const double c = 1.0 / std::sqrt(P.permittivity * P.permeability);
        EMS_CHECK_ARG(c * P.dt < P.h, "time step violates c*dt < h (reference check_params)");
        g = hex_geom(P.grid[0], P.grid[1], P.grid[2]);
        ntot = g.n[0] + g.n[1] + g.n[2];
        fp64 = P.precision == EMS_FP64;
        K = femstab_kmat(P.dt, P.permeability, P.permittivity, P.h, P.stabilization_factor, P.use_ofem);
        init_stream();
        const size_t w = fp64 ? 8 : 4;
        dE.alloc(3 * ntot * w);
        dE.zero(stream);
        dK.alloc(144 * w);
        if (fp64) {
            EMS_CUDA(cudaMemcpyAsync(dK.p, K.data(), 144 * 8, cudaMemcpyHostToDevice, stream));
        } else {
            std::vector<float> kf(K.begin(), K.end());
            EMS_CUDA(cudaMemcpyAsync(dK.p, kf.data(), 144 * 4, cudaMemcpyHostToDevice, stream));
        }
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    size_t comp_off(int c) const { return c == 0 ? 0 : (c == 1 ? g.n[0] : g.n[0] + g.n[1]); }
    long long flat(int c, int i, int j, int k) const { return hex_flat(g, c, i, j, k); }

    // The source statements of one run in the reference's order (point
    // sources x, y, z in insertion order, then the dipoles) and their values
    // per step: point sources s(t) dt^2 / (mu eps h^3), dipole terms
    // w s(t) dt^2 / (mu eps 8).
    template <class T> int upload_sources(int nsteps)
    {
        std::vector<long long> sidx;
        std::vector<double> swt;
        std::vector<int> sop, skind;
        for (int c = 0; c < 3; ++c)
            for (auto &s : srcs)
                if (s[0] == c) { sidx.push_back(flat(c, s[1], s[2], s[3])); swt.push_back(1.0); sop.push_back(1); skind.push_back(0); }
        for (auto &d : dips) {
            const size_t b = sidx.size();
            if (P.use_ofem) {   // fem/fem_simulation.cpp:708-740: one x-edge of cell (i, j+1, k+1)
                sidx.push_back(flat(0, d[0], d[1] + 1, d[2] + 1));
                swt.push_back(8.0);
                sop.push_back(1);
            } else {
                hex_dipole_terms(g, d, P.stabilization_factor, sidx, swt, sop);
            }
            for (size_t q = b; q < sidx.size(); ++q) skind.push_back(1);
        }
        const int ns = (int)sidx.size();
        if (ns == 0) return 0;
        std::vector<double> vals((size_t)ns * std::max(nsteps, 1), 0.0);
        double t = cur_time;
        const double dt = P.dt, mu = P.permeability, eps = P.permittivity, h = P.h;
        for (int st = 0; st < nsteps; ++st) {
            const double f = femstab_source(t, mu, h);
            const double point = f * dt * dt / mu / eps / h / h / h;
            const double temp = f * dt * dt / mu / eps / 8.0;
            for (int s = 0; s < ns; ++s) vals[(size_t)st * ns + s] = skind[s] ? swt[s] * temp : point;
            t += dt;
        }
        d_src_idx.alloc(sidx.size() * 8);
        d_src_op.alloc(sop.size() * 4);
        d_src_val.alloc(vals.size() * 8);
        EMS_CUDA(cudaMemcpyAsync(d_src_idx.p, sidx.data(), sidx.size() * 8, cudaMemcpyHostToDevice, stream));
        EMS_CUDA(cudaMemcpyAsync(d_src_op.p, sop.data(), sop.size() * 4, cudaMemcpyHostToDevice, stream));
        EMS_CUDA(cudaMemcpyAsync(d_src_val.p, vals.data(), vals.size() * 8, cudaMemcpyHostToDevice, stream));
        return ns;
    }

    void upload_receivers(int nsteps)
    {
        const int tf = P.time_frequency;
        nobs = (int)obs_n.size() / 3;
        nsamp = nsteps / tf + 1;
        ncols = 3;
        std::vector<int> start(std::max(nobs, 1), 0);
        std::vector<long long> ridx;
        for (int o = 0; o < nobs; ++o) {
            start[o] = (int)ridx.size();
            for (int c = 0; c < 3; ++c)
                for (auto &q : obs_lists[3 * o + c]) ridx.push_back(flat(c, q[0], q[1], q[2]));
        }
        if (ridx.empty()) ridx.push_back(0);
        std::vector<int> cnt = obs_n;
        if (cnt.empty()) cnt.assign(3, 0);
        d_obs_cnt.alloc(cnt.size() * 4);
        d_obs_start.alloc(start.size() * 4);
        d_obs_idx.alloc(ridx.size() * 8);
        EMS_CUDA(cudaMemcpyAsync(d_obs_cnt.p, cnt.data(), cnt.size() * 4, cudaMemcpyHostToDevice, stream));
        EMS_CUDA(cudaMemcpyAsync(d_obs_start.p, start.data(), start.size() * 4, cudaMemcpyHostToDevice, stream));
        EMS_CUDA(cudaMemcpyAsync(d_obs_idx.p, ridx.data(), ridx.size() * 8, cudaMemcpyHostToDevice, stream));
        d_tr.alloc((size_t)std::max(nobs, 1) * nsamp * 3 * 8);
        d_tr.zero(stream);
    }

    template <class T> void sweep(dim3 grid, T *E0, T *E1, T *E2)
    {
        if (fp64) femstab_sweep_kernel<T, true><<<grid, 128, 0, stream>>>(g, dK.as<T>(), E0, E1, E2);
        else femstab_sweep_kernel<T, false><<<grid, 128, 0, stream>>>(g, dK.as<T>(), E0, E1, E2);
    }

    // fem/fem_simulation.cpp:836-903: per step the update, PEC, then the
    // receivers every tf steps (step counted from 1)
    template <class T> void run_t(int nsteps)
    {
        const int tf = P.time_frequency;
        upload_receivers(nsteps);
        const int ns = upload_sources<T>(nsteps);
        const size_t mx = std::max(g.n[0], std::max(g.n[1], g.n[2]));
        const dim3 grid((unsigned)((mx + 127) / 128), 3);
        long long launches = 0;
        EMS_CUDA(cudaEventRecord(ev0, stream));
        for (int step = 1; step < nsteps + 1; ++step) {
            T *E0 = dE.as<T>() + (size_t)r0 * ntot, *E1 = dE.as<T>() + (size_t)r1 * ntot, *E2 = dE.as<T>() + (size_t)r2 * ntot;
            sweep<T>(grid, E0, E1, E2);
            ++launches;
            if (ns) {
                hex_source_kernel<T><<<1, 32, 0, stream>>>(g, E2, ns, d_src_idx.as<long long>(),
                                                           d_src_val.as<double>() + (size_t)(step - 1) * ns, d_src_op.as<int>(), 1);
                ++launches;
            }
            if (nobs > 0 && step % tf == 0) {
                hex_sample_kernel<T><<<(nobs + 63) / 64, 64, 0, stream>>>(nobs, d_obs_cnt.as<int>(), d_obs_start.as<int>(),
                                                                         d_obs_idx.as<long long>(), E2, d_tr.as<double>(), nsamp,
                                                                         step / tf);
                ++launches;
            }
            cur_time += P.dt;
            r0 = (r0 + 1) % 3; r1 = (r1 + 1) % 3; r2 = (r2 + 1) % 3;
        }
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaEventRecord(ev1, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        float ms = 0;
        EMS_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        last_ms = ms;
        last_launches = launches;
        const size_t ntr = (size_t)std::max(nobs, 1) * nsamp * 3;
        traces.assign(ntr, 0.0);
        EMS_CUDA(cudaMemcpy(traces.data(), d_tr.p, ntr * 8, cudaMemcpyDeviceToHost));
        traces.resize((size_t)nobs * nsamp * 3);
    }

    void run(int nsteps) override
    {
        EMS_CHECK_ARG(nsteps >= 0, "num_steps must be >= 0");
        if (fp64) run_t<double>(nsteps); else run_t<float>(nsteps);
        check_finite({{dE.p, 3 * ntot}}, fp64);
    }

    // which 0..2: E component, its three storage levels in the reference's
    // layout (fem/fem_simulation.cpp:67-72)
    size_t field_size(int which) const override
    {
        if (which < 0 || which > 2) throw Error{EMS_ERR_INVALID_ARGUMENT, "field index must be 0..2 (Ex, Ey, Ez)"};
        return 3 * g.n[which];
    }
    void get_field(int which, double *out) const override
    {
        field_size(which);
        const size_t w = fp64 ? 8 : 4, n = g.n[which];
        for (int l = 0; l < 3; ++l) {
            const char *src = (const char *)dE.p + ((size_t)l * ntot + comp_off(which)) * w;
            if (fp64) {
                EMS_CUDA(cudaMemcpy(out + (size_t)l * n, src, n * 8, cudaMemcpyDeviceToHost));
            } else {
                std::vector<float> tmp(n);
                EMS_CUDA(cudaMemcpy(tmp.data(), src, n * 4, cudaMemcpyDeviceToHost));
                for (size_t q = 0; q < n; ++q) out[(size_t)l * n + q] = tmp[q];
            }
        }
    }
    void set_field(int which, const double *in) override
    {
        field_size(which);
        const size_t w = fp64 ? 8 : 4, n = g.n[which];
        for (int l = 0; l < 3; ++l) {
            char *dst = (char *)dE.p + ((size_t)l * ntot + comp_off(which)) * w;
            if (fp64) {
                EMS_CUDA(cudaMemcpy(dst, in + (size_t)l * n, n * 8, cudaMemcpyHostToDevice));
            } else {
                std::vector<float> tmp(in + (size_t)l * n, in + (size_t)(l + 1) * n);
                EMS_CUDA(cudaMemcpy(dst, tmp.data(), n * 4, cudaMemcpyHostToDevice));
            }
        }
    }
    // fem/fem_simulation.cpp:905-927: the given file name with header
    // time,Ex,Ey,Ez and the stream's default formatting; a second and later
    // receiver get the suffix _<i> (the reference writes every receiver to
    // the same name)
    void save(const char *path) const override
    {
        EMS_CHECK_ARG(path && *path, "file name required");
        for (int o = 0; o < nobs; ++o) {
            std::string fn = path;
            if (o > 0) {
                const size_t dot = fn.rfind('.');
                const std::string suf = "_" + std::to_string(o);
                if (dot == std::string::npos) fn += suf; else fn.insert(dot, suf);
            }
            std::ofstream f(fn);
            if (!f.is_open()) throw Error{EMS_ERR_IO, "cannot open " + fn};
            f << "time,Ex,Ey,Ez" << std::endl;
            for (int j = 0; j < nsamp; ++j) {
                const double *r = &traces[((size_t)o * nsamp + j) * 3];
                f << (size_t)j * P.time_frequency * P.dt << "," << r[0] << "," << r[1] << "," << r[2] << std::endl;
            }
        }
    }
    void reset() override
    {
        dE.zero(stream);
        r0 = 0; r1 = 1; r2 = 2;
        cur_time = 0.0;
        EMS_CUDA(cudaStreamSynchronize(stream));
    }
    void time_dominant(int launches, double *ms, double *bytes, std::string *name) override
    {
        const size_t w = fp64 ? 8 : 4;
        const size_t mx = std::max(g.n[0], std::max(g.n[1], g.n[2]));
        const dim3 grid((unsigned)((mx + 127) / 128), 3);
        // the sweep writes only the E^{n+1} slot, which the next step rewrites
        auto body = [&](auto tag) {
            using T = decltype(tag);
            T *E0 = dE.as<T>() + (size_t)r0 * ntot, *E1 = dE.as<T>() + (size_t)r1 * ntot, *E2 = dE.as<T>() + (size_t)r2 * ntot;
            for (int r = 0; r <= launches; ++r) {
                if (r == 1) EMS_CUDA(cudaEventRecord(ev0, stream));
                sweep<T>(grid, E0, E1, E2);
            }
        };
        if (fp64) body(double()); else body(float());
        EMS_CUDA(cudaGetLastError());
        EMS_CUDA(cudaEventRecord(ev1, stream));
        EMS_CUDA(cudaStreamSynchronize(stream));
        float t = 0;
        EMS_CUDA(cudaEventElapsedTime(&t, ev0, ev1));
        *ms = t / launches;
        *bytes = (double)ntot * w * 3.0;   // read E^{n-1}, E^n; write E^{n+1}
        *name = fp64 ? "femstab_sweep_kernel<double>" : "femstab_sweep_kernel<float>";
    }
};

Sim *make_femstab(const ems_femstab_params *p) { return new FemStabSim(p); }
bool is_femstab(const Sim *s) { return dynamic_cast<const FemStabSim *>(s) != nullptr; }

void femstab_set_source(Sim *s, int comp, const int ijk[3])
{
    auto *f = static_cast<FemStabSim *>(s);
    const int lim[3] = {f->g.gx - (comp == 0), f->g.gy - (comp == 1), f->g.gz - (comp == 2)};
    for (int d = 0; d < 3; ++d) EMS_CHECK_ARG(ijk[d] >= 0 && ijk[d] <= lim[d], "source edge outside the grid");
    f->srcs.push_back({comp, ijk[0], ijk[1], ijk[2]});
}

void femstab_add_dipole(Sim *s, const int ijk[3])
{
    auto *f = static_cast<FemStabSim *>(s);
    EMS_CHECK_ARG(ijk != nullptr, "position required");
    // the dipole touches cells (i, j..j+1, k..k+1)
    EMS_CHECK_ARG(ijk[0] >= 0 && ijk[0] < f->g.gx && ijk[1] >= 0 && ijk[1] + 1 < f->g.gy && ijk[2] >= 0 && ijk[2] + 1 < f->g.gz,
                  "dipole cells outside the grid");
    f->dips.push_back({ijk[0], ijk[1], ijk[2]});
}

void femstab_add_observation(Sim *s, const int *x, int nx, const int *y, int ny, const int *z, int nz)
{
    auto *f = static_cast<FemStabSim *>(s);
    const int *lists[3] = {x, y, z};
    const int cnt[3] = {nx, ny, nz};
    for (int c = 0; c < 3; ++c) {
        EMS_CHECK_ARG(cnt[c] >= 0 && (cnt[c] == 0 || lists[c] != nullptr), "observation list missing");
        const int lim[3] = {f->g.gx - (c == 0), f->g.gy - (c == 1), f->g.gz - (c == 2)};
        std::vector<std::array<int, 3>> v;
        for (int r = 0; r < cnt[c]; ++r) {
            const int *q = lists[c] + 3 * r;
            for (int d = 0; d < 3; ++d) EMS_CHECK_ARG(q[d] >= 0 && q[d] <= lim[d], "observation edge outside the grid");
            v.push_back({q[0], q[1], q[2]});
        }
        f->obs_lists.push_back(v);
        f->obs_n.push_back(cnt[c]);
    }
}

void femstab_element_matrix(const Sim *s, double *K)
{
    const auto *f = static_cast<const FemStabSim *>(s);
    std::memcpy(K, f->K.data(), sizeof(double) * 144);
}

}  // namespace ems
