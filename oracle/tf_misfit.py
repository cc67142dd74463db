"""Time-frequency envelope misfit restated from the published method
(Kristekova, Kristek, Moczo & Day 2006, BSSA 96(5), 1836-1850), used by the
reference's TF_MISFIT_GOF_master pipeline through a prebuilt third-party
executable (no source in the reference; namelist HF_TF-MISFIT_GOF sets
IS_S2_REFERENCE=T, LOCAL_NORM=F).

ORACLE / TEST INFRASTRUCTURE ONLY.  Direct time-domain evaluation of the
continuous wavelet transform with the Morlet wavelet psi(x) = exp(i w0 x)
exp(-x^2/2), w0 = 6 (constant factors dropped: they cancel in the misfit):

    W(t_j, f) = a^{-1/2} sum_i s(t_i) conj(psi((t_i - t_j) / a)) dt,   a = w0 / (2 pi f)

and the single-valued envelope and phase misfits of s against the
reference s_ref

    EM = sqrt( sum_{j,f} (|W(t_j,f)| - |W_ref(t_j,f)|)^2 / sum_{j,f} |W_ref(t_j,f)|^2 ),
    PM = sqrt( sum_{j,f} (|W_ref| dphi / pi)^2 / sum_{j,f} |W_ref|^2 ),
    dphi = Arg W - Arg W_ref wrapped to (-pi, pi].
"""
import numpy as np

W0 = 6.0


def frequencies(fmin, fmax, nf):
    """nf log-spaced frequencies from fmin to fmax."""
    if nf == 1:
        return np.array([fmin])
    return fmin * (fmax / fmin) ** (np.arange(nf) / (nf - 1))


def cwt_morlet(s, dt, freqs):
    """W[f, j] by direct summation (O(nf * n^2); small records only)."""
    n = len(s)
    t = np.arange(n) * dt
    out = np.zeros((len(freqs), n), complex)
    for k, f in enumerate(freqs):
        a = W0 / (2.0 * np.pi * f)
        x = (t[:, None] - t[None, :]) / a           # x[i, j] = (t_i - t_j) / a
        psi = np.exp(1j * W0 * x) * np.exp(-0.5 * x * x)
        out[k] = (np.asarray(s, float)[:, None] * np.conj(psi)).sum(axis=0) * dt / np.sqrt(a)
    return out


def envelope_misfit(s, s_ref, dt, fmin, fmax, nf):
    """EM of s against s_ref (0 when s_ref has no energy in the band)."""
    fr = frequencies(fmin, fmax, nf)
    W, Wr = cwt_morlet(s, dt, fr), cwt_morlet(s_ref, dt, fr)
    den = np.sum(np.abs(Wr) ** 2)
    if den == 0.0:
        return 0.0
    return float(np.sqrt(np.sum((np.abs(W) - np.abs(Wr)) ** 2) / den))


def phase_misfit(s, s_ref, dt, fmin, fmax, nf):
    """PM of s against s_ref (0 when s_ref has no energy in the band)."""
    fr = frequencies(fmin, fmax, nf)
    W, Wr = cwt_morlet(s, dt, fr), cwt_morlet(s_ref, dt, fr)
    den = np.sum(np.abs(Wr) ** 2)
    if den == 0.0:
        return 0.0
    d = np.angle(W) - np.angle(Wr)
    d = np.where(d > np.pi, d - 2 * np.pi, d)
    d = np.where(d <= -np.pi, d + 2 * np.pi, d)
    return float(np.sqrt(np.sum((np.abs(Wr) * d / np.pi) ** 2) / den))
