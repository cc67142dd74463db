"""Trace misfits of libems (host code, no GPU): the L2 misfit and the
time-frequency envelope misfit against the oracle's direct-summation
restatement of the published method, and their trace gradients against
central finite differences."""
import numpy as np
import pytest

import emsolvers_gb300 as ems
from oracle import tf_misfit

DT, NS = 0.05, 201


def _traces(seed, nrec=2):
    rng = np.random.default_rng(seed)
    t = np.arange(NS) * DT
    tr = np.zeros((nrec, NS, 4))
    tr[..., 0] = t
    for r in range(nrec):
        for c in range(3):
            f0, t0, amp = rng.uniform(0.3, 1.2), rng.uniform(3.0, 7.0), rng.uniform(0.5, 2.0)
            tau = t - t0
            tr[r, :, 1 + c] = amp * (1 - 2 * (np.pi * f0 * tau) ** 2) * np.exp(-(np.pi * f0 * tau) ** 2)
    return tr


def test_l2_misfit_and_gradient():
    a, b = _traces(1), _traces(2)
    J, g = ems.trace_misfit(a, b, ems.MISFIT_L2)
    assert J == pytest.approx(0.5 * np.sum((a[..., 1:] - b[..., 1:]) ** 2), rel=1e-14)
    assert np.array_equal(g[..., 1:], a[..., 1:] - b[..., 1:]) and not g[..., 0].any()


@pytest.mark.parametrize("kind", ["envelope", "phase"])
@pytest.mark.parametrize("band", [(0.05, 2.0, 16), (0.2, 4.0, 24)])
def test_tf_misfit_matches_direct_transform(band, kind):
    a, b = _traces(3), _traces(4)
    k, fn = ((ems.MISFIT_TF_ENVELOPE, tf_misfit.envelope_misfit) if kind == "envelope"
             else (ems.MISFIT_TF_PHASE, tf_misfit.phase_misfit))
    J, _ = ems.trace_misfit(a, b, k, band)
    ref = 0.5 * sum(fn(a[r, :, 1 + c], b[r, :, 1 + c], DT, *band) ** 2 for r in range(a.shape[0]) for c in range(3))
    assert J == pytest.approx(ref, rel=1e-6)


@pytest.mark.parametrize("kind", [ems.MISFIT_TF_ENVELOPE, ems.MISFIT_TF_PHASE], ids=["envelope", "phase"])
def test_tf_gradient_matches_finite_differences(kind):
    # directional derivatives along smooth perturbations.  |W| has a cusp
    # where it vanishes and large curvature where it is tiny (the quiet
    # tails of a pulse), so a background of sinusoids across the band keeps
    # the envelopes away from zero; the reference is a delayed, rescaled copy
    # (the inversion regime), so the phase differences stay away from the
    # +-pi wrap where PM is not differentiable
    a = _traces(5)
    t = a[0, :, 0]
    bg = sum(0.05 * np.sin(2 * np.pi * f * t + f) for f in (0.15, 0.4, 0.9, 1.7, 2.6))
    a[..., 1:] += bg[None, :, None]
    b = a.copy()
    b[..., 1:] = 0.9 * a[..., 1:] + 0.1 * np.roll(a[..., 1:], 4, axis=1)
    band = (0.1, 3.0, 20)
    J, g = ems.trace_misfit(a, b, kind, band)
    rng = np.random.default_rng(0)
    for _ in range(4):
        d = np.zeros_like(a)
        for r in range(a.shape[0]):
            for c in range(1, 4):
                d[r, :, c] = np.sin(2 * np.pi * rng.uniform(0.1, 0.8) * t + rng.uniform(0, 6)) * rng.standard_normal()
        h = 1e-5
        fd = (ems.trace_misfit(a + h * d, b, kind, band)[0] - ems.trace_misfit(a - h * d, b, kind, band)[0]) / (2 * h)
        assert np.sum(g * d) == pytest.approx(fd, rel=1e-5)


def test_tf_envelope_misfit_vanishes_for_equal_traces_and_skips_silent_components():
    a = _traces(7)
    J, g = ems.trace_misfit(a, a, ems.MISFIT_TF_ENVELOPE)
    assert J == 0.0 and not g.any()
    b = a.copy()
    b[..., 2] = 0.0    # a silent reference component contributes nothing
    J2, g2 = ems.trace_misfit(a, b, ems.MISFIT_TF_ENVELOPE)
    assert J2 == 0.0 and not g2[..., 2].any()


def test_misfit_rejects_bad_input():
    a = _traces(8)
    with pytest.raises(ems.EmsError):
        ems.trace_misfit(a, a, 7)
    bad = a.copy()
    bad[..., 0] = 0.0
    with pytest.raises(ems.EmsError):
        ems.trace_misfit(bad, bad, ems.MISFIT_TF_ENVELOPE)
