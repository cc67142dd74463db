// Receiver-trace misfits and their gradients with respect to the traces
// (host code, FP64).  They feed the adjoint: dJ/dtraces is the right-hand
// side of ems_tetfem_backward.
//
// L2:  J = 1/2 sum over receivers, samples and components of (E - E_obs)^2.
//
// TF envelope (Kristekova, Kristek, Moczo & Day 2006, BSSA 96(5); the
// criterion the reference's TF_MISFIT_GOF_master pipeline evaluates with a
// prebuilt third-party program, used here with IS_S2_REFERENCE = T and
// LOCAL_NORM = F): each trace component s and its reference s_ref are taken
// to the time-frequency plane by the continuous wavelet transform with the
// analytic Morlet wavelet (omega0 = 6),
//     W(t, f) = (1/sqrt(a)) int s(tau) psi*((tau - t)/a) dtau,  a = omega0/(2 pi f),
// evaluated per frequency through the FFT (Gaussian window
// sqrt(a) exp(-(a omega - omega0)^2 / 2) on omega >= 0, zero padding by 8
// scales of the lowest frequency, so the circular convolution equals the
// linear one to exp(-32)); the envelope difference
// dE(t, f) = |W(t, f)| - |W_ref(t, f)| gives the single-valued envelope
// misfit EM = sqrt(sum dE^2 / sum |W_ref|^2); the phase difference
// dP(t, f) = |W_ref| (Arg W - Arg W_ref) / pi gives the phase misfit PM in
// the same way (components whose reference has no energy in the band are
// skipped).  The constant factors of the transform cancel and are left
// out.  Here J = 1/2 sum EM^2 (or PM^2) over receivers and components
// (smooth where the misfit vanishes, unlike EM itself), and its gradient
// follows through the adjoint A_f^H of the discrete transform at each
// frequency (zero-pad, FFT, window, inverse FFT, crop).
#include <cmath>
#include <complex>
#include <thread>
#include <vector>

#include "ems.h"
#include "ems_internal.hpp"

namespace ems {

namespace {

using cplx = std::complex<double>;

// In-place radix-2 FFT (n a power of two); sign -1 forward, +1 inverse
// (unscaled).
void fft(std::vector<cplx> &a, int sign)
{
    const size_t n = a.size();
    for (size_t i = 1, j = 0; i < n; ++i) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        const double ang = sign * 2.0 * M_PI / (double)len;
        const cplx wl(std::cos(ang), std::sin(ang));
        for (size_t i = 0; i < n; i += len) {
            cplx w(1.0, 0.0);
            for (size_t k = 0; k < len / 2; ++k) {
                cplx u = a[i + k], v = a[i + k + len / 2] * w;
                a[i + k] = u + v;
                a[i + k + len / 2] = u - v;
                w *= wl;
            }
        }
    }
}

struct TfPlan {
    int nsamp = 0;
    size_t n2 = 0;
    std::vector<std::vector<double>> window;   // per frequency, n2 values
};

TfPlan tf_plan(int nsamp, double dt, double fmin, double fmax, int nf)
{
    TfPlan p;
    p.nsamp = nsamp;
    const double omega0 = 6.0;
    const double a_max = omega0 / (2.0 * M_PI * fmin);
    p.n2 = 1;
    while ((double)p.n2 < nsamp + 8.0 * a_max / dt) p.n2 <<= 1;
    p.window.resize(nf);
    for (int k = 0; k < nf; ++k) {
        const double f = nf == 1 ? fmin : fmin * std::pow(fmax / fmin, (double)k / (nf - 1));
        const double a = omega0 / (2.0 * M_PI * f);
        auto &w = p.window[k];
        w.assign(p.n2, 0.0);
        for (size_t m = 0; m < p.n2 / 2; ++m) {
            const double om = 2.0 * M_PI * (double)m / ((double)p.n2 * dt);
            const double x = a * om - omega0;
            w[m] = std::sqrt(a) * std::exp(-0.5 * x * x);
        }
    }
    return p;
}

// W_f for every frequency: nf x nsamp complex values.
void tf_transform(const TfPlan &p, const double *s, std::vector<std::vector<cplx>> &W)
{
    std::vector<cplx> S(p.n2, cplx(0.0, 0.0));
    for (int i = 0; i < p.nsamp; ++i) S[i] = s[i];
    fft(S, -1);
    W.resize(p.window.size());
    std::vector<cplx> tmp(p.n2);
    for (size_t k = 0; k < p.window.size(); ++k) {
        for (size_t m = 0; m < p.n2; ++m) tmp[m] = S[m] * p.window[k][m];
        fft(tmp, +1);
        W[k].resize(p.nsamp);
        for (int i = 0; i < p.nsamp; ++i) W[k][i] = tmp[i] / (double)p.n2;
    }
}

// EM^2 (phase = false) or PM^2 (phase = true) of s against s_ref and, when
// g is given, its half derivative d(X^2 / 2)/ds.
//   envelope: dE = |W| - |W_ref|,           R = dE W / |W|,                 g = Re(A^H R) / N
//   phase:    dP = |W_ref| dphi / pi,       R = |W_ref|^2 dphi W / (pi^2 |W|^2), g = -Im(A^H R) / N
// with dphi = Arg W - Arg W_ref wrapped to (-pi, pi], N = sum |W_ref|^2, and
// A^H R = crop(IFFT(window * FFT(pad(R)))) carrying the 1/n2 of the forward
// transform's inverse FFT.
double tf_misfit(const TfPlan &p, const double *s, const double *sref, double *g, bool phase)
{
    std::vector<std::vector<cplx>> W, Wr;
    tf_transform(p, s, W);
    tf_transform(p, sref, Wr);
    auto dphi = [](const cplx &w, const cplx &wr) {
        double d = std::arg(w) - std::arg(wr);
        if (d > M_PI) d -= 2.0 * M_PI;
        if (d <= -M_PI) d += 2.0 * M_PI;
        return d;
    };
    double num = 0.0, den = 0.0;
    for (size_t k = 0; k < W.size(); ++k)
        for (int i = 0; i < p.nsamp; ++i) {
            const double dX = phase ? std::abs(Wr[k][i]) * dphi(W[k][i], Wr[k][i]) / M_PI
                                    : std::abs(W[k][i]) - std::abs(Wr[k][i]);
            num += dX * dX;
            den += std::norm(Wr[k][i]);
        }
    if (den == 0.0) {   // no reference energy in the band: the component is skipped
        if (g)
            for (int i = 0; i < p.nsamp; ++i) g[i] = 0.0;
        return 0.0;
    }
    if (g) {
        std::vector<double> acc(p.nsamp, 0.0);
        std::vector<cplx> tmp(p.n2);
        for (size_t k = 0; k < W.size(); ++k) {
            std::fill(tmp.begin(), tmp.end(), cplx(0.0, 0.0));
            for (int i = 0; i < p.nsamp; ++i) {
                const double m = std::abs(W[k][i]);
                if (m == 0.0) continue;
                if (phase)
                    tmp[i] = std::norm(Wr[k][i]) * dphi(W[k][i], Wr[k][i]) / (M_PI * M_PI * m * m) * W[k][i];
                else
                    tmp[i] = (m - std::abs(Wr[k][i])) * W[k][i] / m;
            }
            fft(tmp, -1);
            for (size_t m = 0; m < p.n2; ++m) tmp[m] *= p.window[k][m];
            fft(tmp, +1);
            for (int i = 0; i < p.nsamp; ++i) acc[i] += (phase ? -tmp[i].imag() : tmp[i].real()) / (double)p.n2;
        }
        for (int i = 0; i < p.nsamp; ++i) g[i] = acc[i] / den;
    }
    return num / den;
}

}  // namespace

void trace_misfit(int kind, int nobs, int nsamp, const double *tr, const double *obs, double *misfit, double *tg,
                  const double *band)
{
    EMS_CHECK_ARG(nobs >= 0 && nsamp >= 0, "trace sizes must be >= 0");
    EMS_CHECK_ARG((tr && obs && misfit) || nobs * (size_t)nsamp == 0, "traces, observed traces and misfit required");
    const size_t n = (size_t)nobs * nsamp * 4;
    if (n == 0) {
        if (misfit) *misfit = 0.0;
        return;
    }
    if (tg)
        for (size_t i = 0; i < n; ++i) tg[i] = 0.0;
    if (kind == EMS_MISFIT_L2) {
        double J = 0.0;
        for (size_t i = 0; i < n; ++i) {
            if (i % 4 == 0) continue;
            double d = tr[i] - obs[i];
            J += 0.5 * d * d;
            if (tg) tg[i] = d;
        }
        if (misfit) *misfit = J;
        return;
    }
    if (kind != EMS_MISFIT_TF_ENVELOPE && kind != EMS_MISFIT_TF_PHASE)
        throw Error{EMS_ERR_INVALID_ARGUMENT, "unknown misfit kind"};
    const bool phase = kind == EMS_MISFIT_TF_PHASE;
    EMS_CHECK_ARG(nsamp >= 4, "the TF envelope misfit needs at least 4 samples");
    const double dt = tr[4] - tr[0];
    EMS_CHECK_ARG(dt > 0 && std::isfinite(dt), "column 0 must hold increasing sample times");
    double fmin = 4.0 / (nsamp * dt), fmax = 0.25 / dt;
    int nf = 32;
    if (band) {
        fmin = band[0]; fmax = band[1]; nf = (int)band[2];
        EMS_CHECK_ARG(fmin > 0 && fmax >= fmin && nf >= 1, "TF band must be 0 < fmin <= fmax with nf >= 1");
    }
    const TfPlan plan = tf_plan(nsamp, dt, fmin, fmax, nf);
    // one task per (receiver, component), spread over host threads
    const int ntask = nobs * 3;
    std::vector<double> em2(ntask, 0.0);
    unsigned nth = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)ntask));
    std::vector<std::thread> pool;
    std::vector<std::string> fail(nth);
    for (unsigned w = 0; w < nth; ++w)
        pool.emplace_back([&, w] {
            std::vector<double> s(nsamp), sr(nsamp), g(nsamp);
            try {
                for (int task = (int)w; task < ntask; task += (int)nth) {
                    const int r = task / 3, c = task % 3;
                    for (int i = 0; i < nsamp; ++i) {
                        s[i] = tr[((size_t)r * nsamp + i) * 4 + 1 + c];
                        sr[i] = obs[((size_t)r * nsamp + i) * 4 + 1 + c];
                    }
                    em2[task] = tf_misfit(plan, s.data(), sr.data(), tg ? g.data() : nullptr, phase);
                    if (tg)
                        for (int i = 0; i < nsamp; ++i) tg[((size_t)r * nsamp + i) * 4 + 1 + c] = g[i];
                }
            } catch (const Error &e) {
                fail[w] = e.msg;
            }
        });
    for (auto &t : pool) t.join();
    for (auto &m : fail)
        if (!m.empty()) throw Error{EMS_ERR_INVALID_ARGUMENT, m};
    double J = 0.0;
    for (double v : em2) J += 0.5 * v;
    *misfit = J;
}

}  // namespace ems
