// Adams-Bashforth-Moulton hexahedral edge-element solver (fem_abm) on one GPU.
//
// E and H both live on the primal edges of an order-1 hexahedral grid
// (fem_abm/fem_simulation.cpp:66-141, cyclic local edge order); a step is an
// AB2 predictor and an AM3 corrector (278-833) with the element matrix
// K = A + 0.05 Abar (143-246): E is updated with K^T, H with K.  The
// reference scatters element contributions with atomics; here every edge DOF
// gathers them from the (at most four) elements that contain it, in the
// reference's element order, so the FP64 result is bit-identical to the
// serial reference.  Sources, Hertz dipoles (407-481, 758-833), PEC
// (835-943) and receivers (972-1013) follow the reference.
#include <cuda_runtime.h>

#include <cmath>
#include <fstream>
#include <iomanip>

#include "ems_internal.hpp"
#include "hexedge.cuh"

namespace ems {

namespace {

using AbmGeom = HexGeom;

// the four field levels of E and H for one step (ring slots 0..2, scratch 3)
template <class T> struct Lev {
    T *E[4];
    T *H[4];
};

// predictor / corrector right-hand sides (fem_abm 295-319, 484-508, 573-615):
//  AB: Es = (3 H1 - H0) dt/8/eps/h,            Hs = -(3 E1 - E0) dt/8/mu/h
//  AM: Es = (5 H2 + 8 H1 - H0) dt/48/eps/h,    Hs = -(5 E2 + 8 E1 - E0) dt/48/mu/h
template <class T>
__global__ void abm_rhs_kernel(AbmGeom g, Lev<T> L, int am, T dt, T eps, T mu, T h)
{
    T *const *E = L.E, *const *H = L.H;
    const int c = blockIdx.y;
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n[c]) return;
    const size_t o = c == 0 ? 0 : (c == 1 ? g.n[0] : g.n[0] + g.n[1]);
    const T *E0 = E[0] + o, *E1 = E[1] + o, *E2 = E[2] + o, *H0 = H[0] + o, *H1 = H[1] + o, *H2 = H[2] + o;
    T es, hs;
    if (!am) {
        es = dv(dv(dv(ml(sb(ml(T(3), H1[t]), H0[t]), dt), T(8)), eps), h);
        hs = dv(dv(dv(ml(-sb(ml(T(3), E1[t]), E0[t]), dt), T(8)), mu), h);
    } else {
        es = dv(dv(dv(ml(sb(ad(ml(T(5), H2[t]), ml(T(8), H1[t])), H0[t]), dt), T(48)), eps), h);
        hs = dv(dv(dv(ml(-sb(ad(ml(T(5), E2[t]), ml(T(8), E1[t])), E0[t]), dt), T(48)), mu), h);
    }
    E[3][o + t] = es;
    H[3][o + t] = hs;
}

__device__ __forceinline__ bool abm_h_pec(const AbmGeom &g, int c, int i, int j, int k)
{
    if (c == 0) return i == 0 || i == g.gx - 1;
    if (c == 1) return j == 0 || j == g.gy - 1;
    return k == 0 || k == g.gz - 1;
}

// Element sweeps gathered per DOF: E2 = sum_e (K^T Es_e)_r + E1 and
// H2 = sum_e (K Hs_e)_r + H1 over the elements e containing the DOF, in
// increasing element order; with `bc` the PEC of 835-943 is applied.
template <class T, bool EXACT>
__global__ void __launch_bounds__(128) abm_sweep_kernel(AbmGeom g, const T *__restrict__ K, Lev<T> L, int bc)
{
    T *const *E = L.E, *const *H = L.H;
    const int c = blockIdx.y;
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n[c]) return;
    const size_t off[3] = {0, g.n[0], g.n[0] + g.n[1]};
    int i, j, k;
    hex_coords(g, c, t, i, j, k);
    // candidate cells: offsets (a0, a1) on the two transverse axes of the
    // cyclic order, local q = a0 + 2 a1, visited in increasing element index
    T acc_e = 0, acc_h = 0;
    const int ord[3][4] = {{3, 2, 1, 0}, {3, 1, 2, 0}, {3, 2, 1, 0}};
    for (int oi = 0; oi < 4; ++oi) {
        const int qq = ord[c][oi];
        int a0 = qq & 1, a1 = qq >> 1;
        int ci = i, cj = j, ck = k;
        if (c == 0) { cj -= a0; ck -= a1; }
        else if (c == 1) { ck -= a0; ci -= a1; }
        else { ci -= a0; cj -= a1; }
        if (ci < 0 || cj < 0 || ck < 0 || ci >= g.gx || cj >= g.gy || ck >= g.gz) continue;
        const int r = 4 * c + qq;
        T te = 0, th = 0;
        for (int m = 0; m < 12; ++m) {
            int mc = m >> 2, mq = m & 3;
            size_t idx = off[mc] + hex_edge(g, mc, ci, cj, ck, mq);
            T es = E[3][idx], hs = H[3][idx];
            if (EXACT) {
                te = ad(te, ml(K[m * 12 + r], es));
                th = ad(th, ml(K[r * 12 + m], hs));
            } else {
                te = fma(K[m * 12 + r], es, te);
                th = fma(K[r * 12 + m], hs, th);
            }
        }
        acc_e = EXACT ? ad(acc_e, te) : acc_e + te;
        acc_h = EXACT ? ad(acc_h, th) : acc_h + th;
    }
    T e2 = EXACT ? ad(acc_e, E[1][off[c] + t]) : acc_e + E[1][off[c] + t];
    T h2 = EXACT ? ad(acc_h, H[1][off[c] + t]) : acc_h + H[1][off[c] + t];
    if (bc) {
        if (hex_e_pec(g, c, i, j, k)) e2 = 0;
        if (abm_h_pec(g, c, i, j, k)) h2 = 0;
    }
    E[2][off[c] + t] = e2;
    H[2][off[c] + t] = h2;
}

double abm_source(double t, double h)
{
    const double f0 = 1.0e9;
    return -4.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) *
           std::exp(-2.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) * (t - 1.0 / f0)) / h / h / h * 0.001;
}

}  // namespace

struct AbmSim : Sim {
    ems_hexfem_params P;
    std::string kdir;
    AbmGeom g{};
    bool fp64;
    size_t ntot;
    DevBuf dE, dH, dK, d_src_idx, d_src_val, d_src_op, d_obs_cnt, d_obs_start, d_obs_idx, d_tr;
    std::vector<std::array<int, 4>> srcs;          // comp, i, j, k
    std::vector<std::array<int, 3>> dips;          // x-directed Hertz dipoles
    std::vector<std::vector<std::array<int, 3>>> obs_lists;
    std::vector<int> obs_n;
    int r0 = 0, r1 = 1, r2 = 2;
    double cur_time = 0.0;
    static constexpr double kSF = 0.05;

    explicit AbmSim(const ems_hexfem_params *p) : Sim(Kind::HEXFEM), P(*p)
    {
        kdir = P.kmat_dir ? P.kmat_dir : "kmat";
        P.kmat_dir = nullptr;
        EMS_CHECK_ARG(P.order == 1, "the Adams-Bashforth-Moulton solver is order 1");
        EMS_CHECK_ARG(P.precision == EMS_FP64 || P.precision == EMS_FP32, "precision must be EMS_FP64 or EMS_FP32");
        EMS_CHECK_ARG(P.h > 0 && P.dt > 0 && P.permittivity > 0 && P.permeability > 0, "h, dt, eps, mu must be positive");
        EMS_CHECK_ARG(P.time_frequency > 0, "time_frequency must be positive");
        EMS_CHECK_ARG(P.grid[0] >= 2 && P.grid[1] >= 2 && P.grid[2] >= 2, "need at least two cells per direction");
        double c = 1.0 / std::sqrt(P.permittivity * P.permeability);
        EMS_CHECK_ARG(c * P.dt < P.h, "time step violates c*dt < h (reference check_params)");
        g = hex_geom(P.grid[0], P.grid[1], P.grid[2]);
        ntot = g.n[0] + g.n[1] + g.n[2];
        fp64 = P.precision == EMS_FP64;
        // K = A + 0.05 Abar (fem_abm/fem_simulation.cpp:143-246)
        auto L = load_matrix_csv(kdir + "/lamped1.csv");
        if (L.size() != 12) throw Error{EMS_ERR_IO, kdir + "/lamped1.csv: expected 12 rows"};
        for (auto &r : L)
            if (r.size() != 12) throw Error{EMS_ERR_IO, kdir + "/lamped1.csv: expected 12 columns"};
        static const double cx[12] = {0, 0, 0, 0, 0.5, -0.5, 0.5, -0.5, -0.5, -0.5, 0.5, 0.5};
        static const double cy[12] = {-0.5, -0.5, 0.5, 0.5, 0, 0, 0, 0, 0.5, -0.5, 0.5, -0.5};
        static const double cz[12] = {0.5, -0.5, 0.5, -0.5, -0.5, -0.5, 0.5, 0.5, 0, 0, 0, 0};
        int perm[12];
        for (int q = 0; q < 4; ++q) { perm[q] = q; perm[8 + q] = 8 + q; perm[4 + q] = 4 + (q / 2) + 2 * (q % 2); }
        std::vector<double> K(144);
        for (int r = 0; r < 12; ++r)
            for (int cc = 0; cc < 12; ++cc) {
                const double *cr = r < 4 ? cx : r < 8 ? cy : cz;
                K[r * 12 + cc] = cr[cc] + kSF * L[perm[r]][perm[cc]];
            }
        init_stream();
        size_t w = fp64 ? 8 : 4;
        dE.alloc(4 * ntot * w); dE.zero(stream);
        dH.alloc(4 * ntot * w); dH.zero(stream);
        if (fp64) {
            dK.alloc(144 * 8);
            EMS_CUDA(cudaMemcpyAsync(dK.p, K.data(), 144 * 8, cudaMemcpyHostToDevice, stream));
        } else {
            std::vector<float> kf(K.begin(), K.end());
            dK.alloc(144 * 4);
            EMS_CUDA(cudaMemcpyAsync(dK.p, kf.data(), 144 * 4, cudaMemcpyHostToDevice, stream));
        }
        EMS_CUDA(cudaStreamSynchronize(stream));
    }

    size_t comp_off(int c) const { return c == 0 ? 0 : (c == 1 ? g.n[0] : g.n[0] + g.n[1]); }
    long long flat(int c, int i, int j, int k) const { return hex_flat(g, c, i, j, k); }
    // device layout: [level][component], 4 levels of ntot values; the ring
    // maps the logical levels n-1, n, n+1 to storage slots
    template <class T> Lev<T> levels(int ring[3]) const
    {
        Lev<T> L;
        for (int l = 0; l < 3; ++l) { L.E[l] = dE.as<T>() + (size_t)ring[l] * ntot; L.H[l] = dH.as<T>() + (size_t)ring[l] * ntot; }
        L.E[3] = dE.as<T>() + 3 * ntot;
        L.H[3] = dH.as<T>() + 3 * ntot;
        return L;
    }

    template <class T> void run_t(int nsteps)
    {
        const int tf = P.time_frequency;
        nobs = (int)obs_n.size() / 3;
        nsamp = nsteps / tf + 1;
        ncols = 3;
        // receivers
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
        size_t ntr = (size_t)std::max(nobs, 1) * nsamp * 3;
        d_tr.alloc(ntr * 8);
        d_tr.zero(stream);
        // source statement lists per phase: point sources then dipoles
        std::vector<long long> sidx;
        std::vector<double> swt;
        std::vector<int> sop, skind;    // kind 0 = point, 1 = dipole
        for (int c = 0; c < 3; ++c)
            for (auto &s : srcs)
                if (s[0] == c) { sidx.push_back(flat(c, s[1], s[2], s[3])); swt.push_back(1.0); sop.push_back(0); skind.push_back(0); }
        for (auto &d : dips) {
            size_t b = sidx.size();
            hex_dipole_terms(g, d, kSF, sidx, swt, sop);
            for (size_t q = b; q < sidx.size(); ++q) skind.push_back(1);
        }
        const int ns = (int)sidx.size();
        std::vector<double> vals((size_t)std::max(ns, 1) * 2 * std::max(nsteps, 1), 0.0);
        {
            double t = cur_time;
            const double h = P.h, dt = P.dt, eps = P.permittivity;
            for (int st = 0; st < nsteps; ++st) {
                double ab_p = (3.0 * abm_source(t, h) - abm_source(t - dt, h)) * dt / 2.0 / eps / h / h / h;
                double ab_d = -(3.0 * abm_source(t, h) - abm_source(t - dt, h)) * dt / 16.0 / eps;
                double am_p = (5.0 * abm_source(t + dt, h) + 8.0 * abm_source(t, h) - abm_source(t - dt, h)) * dt / 12.0 / eps / h / h / h;
                double am_d = -(5.0 * abm_source(t + dt, h) + 8.0 * abm_source(t, h) - abm_source(t - dt, h)) * dt / 96.0 / eps;
                for (int s = 0; s < ns; ++s) {
                    vals[((size_t)st * 2 + 0) * ns + s] = skind[s] ? swt[s] * ab_d : ab_p;
                    vals[((size_t)st * 2 + 1) * ns + s] = skind[s] ? swt[s] * am_d : am_p;
                }
                t += dt;
            }
        }
        if (ns) {
            d_src_idx.alloc(sidx.size() * 8);
            d_src_op.alloc(sop.size() * 4);
            d_src_val.alloc(vals.size() * 8);
            EMS_CUDA(cudaMemcpyAsync(d_src_idx.p, sidx.data(), sidx.size() * 8, cudaMemcpyHostToDevice, stream));
            EMS_CUDA(cudaMemcpyAsync(d_src_op.p, sop.data(), sop.size() * 4, cudaMemcpyHostToDevice, stream));
            EMS_CUDA(cudaMemcpyAsync(d_src_val.p, vals.data(), vals.size() * 8, cudaMemcpyHostToDevice, stream));
        }
        const bool exact = fp64;
        size_t mx = std::max(g.n[0], std::max(g.n[1], g.n[2]));
        dim3 grid((unsigned)((mx + 127) / 128), 3);
        long long launches = 0;
        EMS_CUDA(cudaEventRecord(ev0, stream));
        for (int step = 1; step < nsteps + 1; ++step) {
            int ring[3] = {r0, r1, r2};
            Lev<T> L = levels<T>(ring);
            T *const *Ep = L.E;
            const T dt = (T)P.dt, eps = (T)P.permittivity, mu = (T)P.permeability, h = (T)P.h;
            abm_rhs_kernel<T><<<grid, 128, 0, stream>>>(g, L, 0, dt, eps, mu, h);
            if (exact) abm_sweep_kernel<T, true><<<grid, 128, 0, stream>>>(g, dK.as<T>(), L, 0);
            else abm_sweep_kernel<T, false><<<grid, 128, 0, stream>>>(g, dK.as<T>(), L, 0);
            launches += 2;
            if (ns) {
                hex_source_kernel<T><<<1, 32, 0, stream>>>(g, Ep[2], ns, d_src_idx.as<long long>(),
                                                           d_src_val.as<double>() + ((size_t)(step - 1) * 2 + 0) * ns, d_src_op.as<int>(), 0);
                ++launches;
            }
            abm_rhs_kernel<T><<<grid, 128, 0, stream>>>(g, L, 1, dt, eps, mu, h);
            if (exact) abm_sweep_kernel<T, true><<<grid, 128, 0, stream>>>(g, dK.as<T>(), L, 1);
            else abm_sweep_kernel<T, false><<<grid, 128, 0, stream>>>(g, dK.as<T>(), L, 1);
            launches += 2;
            if (ns) {
                hex_source_kernel<T><<<1, 32, 0, stream>>>(g, Ep[2], ns, d_src_idx.as<long long>(),
                                                           d_src_val.as<double>() + ((size_t)(step - 1) * 2 + 1) * ns, d_src_op.as<int>(), 1);
                ++launches;
            }
            if (nobs > 0 && step % tf == 0) {
                hex_sample_kernel<T><<<(nobs + 63) / 64, 64, 0, stream>>>(nobs, d_obs_cnt.as<int>(), d_obs_start.as<int>(),
                                                                         d_obs_idx.as<long long>(), Ep[2], d_tr.as<double>(), nsamp, step / tf);
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
        traces.assign(ntr, 0.0);
        EMS_CUDA(cudaMemcpy(traces.data(), d_tr.p, ntr * 8, cudaMemcpyDeviceToHost));
        traces.resize((size_t)nobs * nsamp * 3);
    }

    void run(int nsteps) override
    {
        EMS_CHECK_ARG(nsteps >= 0, "num_steps must be >= 0");
        if (fp64) run_t<double>(nsteps); else run_t<float>(nsteps);
        check_finite({{dE.p, 3 * ntot}, {dH.p, 3 * ntot}}, fp64);   // the three ring levels (the scratch level is not state)
    }

    // which 0..2: E components (4 levels each, the reference's layout per
    // component); 3..5: H components.
    size_t field_size(int which) const override
    {
        if (which < 0 || which > 5) throw Error{EMS_ERR_INVALID_ARGUMENT, "field index must be 0..5 (Ex,Ey,Ez,Hx,Hy,Hz)"};
        return 4 * g.n[which % 3];
    }
    void get_field(int which, double *out) const override
    {
        field_size(which);
        int c = which % 3;
        const DevBuf &b = which < 3 ? dE : dH;
        size_t w = fp64 ? 8 : 4;
        for (int l = 0; l < 4; ++l) {
            size_t src = ((size_t)l * ntot + comp_off(c)) * w;
            if (fp64) {
                EMS_CUDA(cudaMemcpy(out + (size_t)l * g.n[c], (char *)b.p + src, g.n[c] * 8, cudaMemcpyDeviceToHost));
            } else {
                std::vector<float> tmp(g.n[c]);
                EMS_CUDA(cudaMemcpy(tmp.data(), (char *)b.p + src, g.n[c] * 4, cudaMemcpyDeviceToHost));
                for (size_t q = 0; q < g.n[c]; ++q) out[(size_t)l * g.n[c] + q] = tmp[q];
            }
        }
    }
    void set_field(int which, const double *in) override
    {
        field_size(which);
        int c = which % 3;
        DevBuf &b = which < 3 ? dE : dH;
        size_t w = fp64 ? 8 : 4;
        for (int l = 0; l < 4; ++l) {
            size_t dst = ((size_t)l * ntot + comp_off(c)) * w;
            if (fp64) {
                EMS_CUDA(cudaMemcpy((char *)b.p + dst, in + (size_t)l * g.n[c], g.n[c] * 8, cudaMemcpyHostToDevice));
            } else {
                std::vector<float> tmp(in + (size_t)l * g.n[c], in + (size_t)(l + 1) * g.n[c]);
                EMS_CUDA(cudaMemcpy((char *)b.p + dst, tmp.data(), g.n[c] * 4, cudaMemcpyHostToDevice));
            }
        }
    }
    // fem_abm/fem_simulation.cpp:1021-1045: results_<i>_<dt>_<h>_<N>.csv
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
    void reset() override
    {
        dE.zero(stream);
        dH.zero(stream);
        r0 = 0; r1 = 1; r2 = 2;
        cur_time = 0.0;
        EMS_CUDA(cudaStreamSynchronize(stream));
    }
    void time_dominant(int launches, double *ms, double *bytes, std::string *name) override
    {
        size_t w = fp64 ? 8 : 4;
        int ring[3] = {r0, r1, r2};
        auto body = [&](auto tag) {
            using T = decltype(tag);
            Lev<T> L = levels<T>(ring);
            T *const *Ep = L.E, *const *Hp = L.H;
            size_t mx = std::max(g.n[0], std::max(g.n[1], g.n[2]));
            dim3 grid((unsigned)((mx + 127) / 128), 3);
            // a sweep without BC changes only the level-2 buffers, which the step rewrites
            DevBuf s2E, s2H;
            s2E.alloc(ntot * w); s2H.alloc(ntot * w);
            EMS_CUDA(cudaMemcpyAsync(s2E.p, Ep[2], ntot * w, cudaMemcpyDeviceToDevice, stream));
            EMS_CUDA(cudaMemcpyAsync(s2H.p, Hp[2], ntot * w, cudaMemcpyDeviceToDevice, stream));
            for (int r = 0; r <= launches; ++r) {
                if (r == 1) EMS_CUDA(cudaEventRecord(ev0, stream));
                if (fp64) abm_sweep_kernel<T, true><<<grid, 128, 0, stream>>>(g, dK.as<T>(), L, 0);
                else abm_sweep_kernel<T, false><<<grid, 128, 0, stream>>>(g, dK.as<T>(), L, 0);
            }
            EMS_CUDA(cudaEventRecord(ev1, stream));
            EMS_CUDA(cudaMemcpyAsync(Ep[2], s2E.p, ntot * w, cudaMemcpyDeviceToDevice, stream));
            EMS_CUDA(cudaMemcpyAsync(Hp[2], s2H.p, ntot * w, cudaMemcpyDeviceToDevice, stream));
            EMS_CUDA(cudaStreamSynchronize(stream));
        };
        if (fp64) body(double()); else body(float());
        float t = 0;
        EMS_CUDA(cudaEventElapsedTime(&t, ev0, ev1));
        *ms = t / launches;
        // read Es, Hs, E1, H1; write E2, H2
        *bytes = (double)ntot * w * 6.0;
        *name = fp64 ? "abm_sweep_kernel<double>" : "abm_sweep_kernel<float>";
    }
};

Sim *make_abm(const ems_hexfem_params *p) { return new AbmSim(p); }

void abm_set_source(Sim *s, int comp, const int ijk[3])
{
    auto *f = static_cast<AbmSim *>(s);
    int lim[3] = {f->g.gx - (comp == 0), f->g.gy - (comp == 1), f->g.gz - (comp == 2)};
    for (int d = 0; d < 3; ++d) EMS_CHECK_ARG(ijk[d] >= 0 && ijk[d] <= lim[d], "source edge outside the grid");
    f->srcs.push_back({comp, ijk[0], ijk[1], ijk[2]});
}

void abm_add_dipole(Sim *s, const int ijk[3])
{
    auto *f = static_cast<AbmSim *>(s);
    EMS_CHECK_ARG(ijk != nullptr, "position required");
    // the dipole touches cells (i, j..j+1, k..k+1)
    EMS_CHECK_ARG(ijk[0] >= 0 && ijk[0] < f->g.gx && ijk[1] >= 0 && ijk[1] + 1 < f->g.gy && ijk[2] >= 0 && ijk[2] + 1 < f->g.gz,
                  "dipole cells outside the grid");
    f->dips.push_back({ijk[0], ijk[1], ijk[2]});
}

void abm_add_observation(Sim *s, const int *x, int nx, const int *y, int ny, const int *z, int nz)
{
    auto *f = static_cast<AbmSim *>(s);
    const int *lists[3] = {x, y, z};
    int cnt[3] = {nx, ny, nz};
    for (int c = 0; c < 3; ++c) {
        EMS_CHECK_ARG(cnt[c] >= 0 && (cnt[c] == 0 || lists[c] != nullptr), "observation list missing");
        int lim[3] = {f->g.gx - (c == 0), f->g.gy - (c == 1), f->g.gz - (c == 2)};
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

bool is_abm(const Sim *s) { return dynamic_cast<const AbmSim *>(s) != nullptr; }

}  // namespace ems
