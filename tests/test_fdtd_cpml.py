"""Physical pin of the CPML (Roden & Gedney 2000; the reference has none, so
the oracle's CPML is checked against physics, not against the reference).

A Ricker pulse from a point source in a box truncated by a CPML is compared
with the same pulse in a box large enough that no echo from its PEC walls
reaches the receiver within the window: their difference is what the CPML
reflects.  Normal, oblique (edge) and corner incidence; the reflection must
sit far below the PEC wall's and fall as the layer thickens.  The oracle is
bit-identical to the GPU path in FP64 (test_fdtd_gpu.py), so this pins both."""
import numpy as np
import pytest

import oracle

H, C0 = 1e-3, 299792458.0
EPS0, MU0 = 8.854187817e-12, 1.25663706212e-6
DT = 0.99 * H / (C0 * np.sqrt(3))
F0 = C0 / (15 * H)                 # 15 cells per wavelength
WINDOW = 160                       # steps: the direct pulse and the CPML echo pass the receivers
BIG = 104                          # PEC walls 52 cells from the source: their echo arrives after the window


def _traces(n, src, recs, steps, pml):
    obs = [([], [], [r]) for r in recs]
    tr, _ = oracle.fdtd_run(n, n, n, H, DT, EPS0, MU0, 1, steps, [(2, src, 1, F0, 1.0)], obs, pml=pml)
    return tr[:, :, 2]


def _reflection(interior, L, pml, recs_rel):
    """Relative L2 difference of the Ez traces (CPML box against the large
    box) at receivers given relative to the source."""
    n = interior + 2 * L
    c = n // 2
    recs = [(c + a, c + b, c + d) for a, b, d in recs_rel]
    small = _traces(n, (c, c, c), recs, WINDOW, pml)
    off = (BIG - n) // 2
    big = _traces(BIG, (c + off,) * 3, [tuple(v + off for v in r) for r in recs], WINDOW, None)
    assert np.abs(big).max() > 0
    return [np.linalg.norm(small[q] - big[q]) / np.linalg.norm(big[q]) for q in range(len(recs))]


# 3 cells in front of the CPML along z (normal), 8 cells along x and y
# (oblique onto an edge region), 7 cells along each axis (corner)
RECS = [(0, 0, 9), (8, 8, 0), (7, 7, 7)]


def test_cpml_reflects_far_less_than_a_pec_wall():
    refl = _reflection(24, 8, dict(cells=8, m=3.0, R0=1e-6), RECS)
    pec = _reflection(40, 0, None, RECS)          # the same box with PEC walls where the CPML was
    assert max(refl) < 1e-3, refl                  # measured 1.8e-4 .. 2.4e-4 (below -70 dB)
    assert min(pec) > 0.5, pec


def test_cpml_reflection_falls_as_the_layer_thickens():
    r = [_reflection(24, L, dict(cells=L, m=3.0, R0=1e-6), RECS[:2]) for L in (4, 8, 12)]
    for q in range(2):
        assert r[0][q] > 10 * r[1][q] > 10 * 5 * r[2][q], r   # measured 3.7e-2, 2.3e-4, 2.9e-5 (normal)
    assert max(r[2]) < 1e-4


def test_complex_frequency_shifted_cpml_absorbs():
    # kappa_max > 1 and alpha_max > 0 (complex frequency shift): alpha lowers
    # the absorption of low frequencies, so the bound is looser
    refl = _reflection(24, 8, dict(cells=8, m=3.0, R0=1e-6, kmax=5.0, amax=0.05), RECS)
    assert max(refl) < 1e-2, refl                  # measured 4.4e-3 .. 5.9e-3
