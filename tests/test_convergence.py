"""The resolution-study driver (emsolvers_gb300.convergence): order fits in
the form of the reference's a_plot.py, EM/PM tables in the form of a.py, on
synthetic traces whose error shrinks like dx^2 (CPU), and on tetrahedral
runs of one cavity at growing resolution (GPU)."""
import numpy as np
import pytest

import emsolvers_gb300 as ems
from emsolvers_gb300 import convergence


def _ricker(t, f0, t0):
    a = (np.pi * f0 * (t - t0)) ** 2
    return (1 - 2 * a) * np.exp(-a)


def _trace(t, shift, scale=1.0):
    tr = np.zeros((1, len(t), 4))
    tr[0, :, 0] = t
    tr[0, :, 1] = scale * _ricker(t, 0.8, 4.0 + shift)
    tr[0, :, 3] = 0.5 * scale * _ricker(t, 0.5, 5.0 + shift)
    return tr


def test_order_fit_matches_a_plot_definition():
    res = np.arange(1, 9)
    y = 3.0 * (0.01 / res) ** 2
    assert convergence.convergence_order(y, 0.01, res) == pytest.approx(2.0, rel=1e-12)


def test_study_recovers_second_order_phase_convergence(tmp_path):
    t = np.arange(400) * 0.05
    ref = _trace(t, 0.0)[0]
    table, orders = convergence.convergence_study(lambda n: _trace(t, 0.2 / n ** 2), range(1, 9), ref,
                                                 tf_band=(0.1, 3.0, 24), csv_path=tmp_path / "c.csv")
    assert table.shape == (8, 6)
    assert np.all(table[:, 2:4] == 0.0)          # silent Ey: skipped
    assert np.all(np.diff(table[:, 1]) < 0)      # PM of Ex falls with n
    assert orders["ExPM"] == pytest.approx(2.0, abs=0.15)
    assert orders["EzPM"] == pytest.approx(2.0, abs=0.15)
    lines = (tmp_path / "c.csv").read_text().splitlines()
    assert lines[0] == ",".join(convergence.COLUMNS) and len(lines) == 9


def test_identical_trace_has_zero_misfits():
    t = np.arange(300) * 0.05
    tr = _trace(t, 0.0)[0]
    assert convergence.component_misfits(tr, tr) == [0.0] * 6


@pytest.mark.gpu
def test_tetrahedral_cavity_converges():
    L, C0 = 0.01, 299792458.0
    f0 = C0 / (L / 2)                                  # wavelength = half the cavity

    def run(n):
        s = ems.TetFemSimulation((n, n, n), L / n, 1, ems.SYMP4, ems.FP64, dt=0.0, cfl_fraction=0.5)
        s.set_material(np.ones(6 * n ** 3))
        s.add_dipole((0.43 * L, 0.51 * L, 0.47 * L), (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0)
        s.add_receiver((0.7 * L, 0.45 * L, 0.55 * L))
        dt, _ = s.time_step()
        s.run(int(round(6.0 / f0 / dt)))
        return s.traces()

    ref = run(24)[0]
    band = (0.2 * f0, 3.0 * f0, 24)
    table, orders = convergence.convergence_study(run, [6, 8, 12], ref, dx=L, tf_band=band)
    em_z = table[:, 4]
    assert em_z[-1] < em_z[0]
    assert orders["EzEM"] > 0.5
