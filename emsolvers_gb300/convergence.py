"""Resolution study in the form of the reference's validation workflow
(TF_MISFIT_GOF_master/output/a.py and a_plot.py): the same receiver is
simulated at resolutions n = 1, 2, ..., its traces are compared with a
reference signal by the single-valued TF envelope and phase misfits (EM, PM
per component), and a convergence order is fitted on log-log axes from the
first and last resolutions (cell size dx / n).

The misfits come from ``ems_trace_misfit`` (host code of libems); the runs are
whatever the caller's ``run(n)`` does, e.g. a TetFemSimulation or a
HexFemSimulation at n times the base resolution.
"""
import csv

import numpy as np

from .solvers import MISFIT_TF_ENVELOPE, MISFIT_TF_PHASE, trace_misfit

COLUMNS = ["ExEM", "ExPM", "EyEM", "EyPM", "EzEM", "EzPM"]


def _resample(trace, times):
    """trace [nsamp, 4] (t, Ex, Ey, Ez) linearly interpolated onto `times`."""
    out = np.zeros((len(times), 4))
    out[:, 0] = times
    for c in range(3):
        out[:, 1 + c] = np.interp(times, trace[:, 0], trace[:, 1 + c], left=0.0, right=0.0)
    return out


def component_misfits(trace, reference, tf_band=None):
    """EM and PM of each component of one receiver trace ([nsamp, 4]) against
    the reference trace on its time grid: [ExEM, ExPM, EyEM, EyPM, EzEM, EzPM]
    (components whose reference is silent give 0)."""
    ref = np.asarray(reference, dtype=np.float64)
    tr = _resample(np.asarray(trace, dtype=np.float64), ref[:, 0])
    row = []
    for c in range(3):
        one_tr = np.zeros((1,) + tr.shape)
        one_ref = np.zeros((1,) + ref.shape)
        one_tr[0, :, 0] = one_ref[0, :, 0] = ref[:, 0]
        one_tr[0, :, 1 + c] = tr[:, 1 + c]
        one_ref[0, :, 1 + c] = ref[:, 1 + c]
        for kind in (MISFIT_TF_ENVELOPE, MISFIT_TF_PHASE):
            J, _ = trace_misfit(one_tr, one_ref, kind, tf_band)   # J = EM^2 / 2 (or PM^2 / 2)
            row.append(float(np.sqrt(2.0 * J)))
    return row


def convergence_order(values, dx, resolutions):
    """Order from the first and last points of value(dx / n), as a_plot.py does."""
    x = dx / np.asarray(resolutions, dtype=np.float64)
    y = np.asarray(values, dtype=np.float64)
    if y[0] <= 0 or y[-1] <= 0:
        return float("nan")
    return float((np.log(y[-1]) - np.log(y[0])) / (np.log(x[-1]) - np.log(x[0])))


def convergence_study(run, resolutions, reference, dx=0.01, receiver=0, tf_band=None, csv_path=None):
    """Runs `run(n)` for every resolution (it returns the traces of the run,
    [nobs, nsamp, 4]), computes the EM/PM table of `receiver` against the
    reference trace ([nsamp, 4]) and the order of every column.  Writes the
    table in the layout of output/a.py (columns ExEM ... EzPM, one row per
    resolution) when csv_path is given.  Returns (table, orders)."""
    table = np.array([component_misfits(run(n)[receiver], reference, tf_band) for n in resolutions])
    orders = {col: convergence_order(table[:, i], dx, resolutions) for i, col in enumerate(COLUMNS)}
    if csv_path is not None:
        with open(csv_path, "w", newline="") as f:
            w = csv.writer(f)
            w.writerow(COLUMNS)
            w.writerows(table.tolist())
    return table, orders
