"""Benchmark of the GB300 Maxwell engine on its headline workload.

Workload (one bench step = one complete forward solve): lowest-order Nedelec
FEM on a 32^3 cube of unit cells, each split into 6 tetrahedra (196,608 tets,
238,688 edges), eps_r i.i.d. U[1,4] per tet (seeded), mu_r = 1, sigma = 0, PEC
walls, 4th-order symplectic integrator, dt = 0.9 x the stability limit, 2000
time steps, one Ricker dipole with f0 set for 10 cells per wavelength, 8
receivers, FP32 fields.  Metric: DOF-updates/s (edges x time steps / time).

`value`   device time of the solve (CUDA events on the solver's stream),
          inputs resident, L2 flushed between solves.
`e2e`     the same solve through the C ABI from host buffers: material upload,
          FP64 mass-block setup and stability limit, time loop, trace download.
`roofline` the dominant kernel (tet_step_kernel, the fused kick + drift of one
          substep) timed alone on the same state, alternating the two U
          buffers as the time loop does.
`cpu_baseline` the FP64 oracle on the host cores over a bounded sample.
A secondary object `fdtd_512` times the 512^3 FP32 Yee update with a 10-cell
CPML (HBM-bound) for a bounded number of steps; `batch64` times 64 batched
shots of uneven size (FP32) against the per-shot FP64 GPU path; `adjoint16`
times the forward + adjoint misfit gradient of 16 shots on a 48^3 x 6 tet
cube (FP32 batched against the per-shot FP64 GPU path).

`--impl reference` times the FP64 CPU oracle (the reference has no
tetrahedral solver; this is the restated algorithm) with all host threads.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

C0 = 299792458.0
N = 32
STEPS_PER_SOLVE = 2000
H = 1e-3
SEED = 2024
# DRAM bytes (read + write) of one step launch on the headline mesh, from
# the ncu capture summarised in profiles/tet_slot_tet32_symp4.md
TRAFFIC_PER_LAUNCH = 7115776


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


def workload():
    ntet = 6 * N ** 3
    rng = np.random.default_rng(SEED)
    eps = rng.uniform(1.0, 4.0, ntet)
    f0 = C0 / (10 * H * np.sqrt(eps.mean()))         # 10 cells per wavelength at the mean speed
    src = (np.array([0.5, 0.5, 0.5]) * N + np.array([0.13, 0.27, 0.41])) * H
    ang = np.arange(8) * np.pi / 4
    recs = [np.array([N / 2 + 10 * np.cos(a), N / 2 + 10 * np.sin(a), N / 2 + 0.3]) * H for a in ang]
    return eps, f0, src, recs


def n_edges(n):
    return 3 * n * (n + 1) ** 2 + 3 * n ** 2 * (n + 1) + n ** 3


def n_dofs2(n):
    """DOFs of the second-order tetrahedra on an n^3 cube: 2 per edge, 2 per
    face (6 face types span two axes, 6 span three)."""
    return 2 * (n_edges(n) + 6 * n ** 2 * (n + 1) + 6 * n ** 3)


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [l.split(",") for l in open(self.f.name).read().splitlines() if l.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) >= 9 for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def flush_l2(buf):
    buf.zero_()


def cpu_oracle_rate(steps, threads):
    """FP64 oracle on `steps` time steps of the same case: DOF-updates/s."""
    import oracle
    os.environ["OMP_NUM_THREADS"] = str(threads)
    eps, f0, src, recs = workload()
    ts = H / C0
    lam = None
    dtn = 0.9 * oracle.stability_constant(oracle.SYMP4) / np.sqrt(oracle.tet_lambda_max((N, N, N), eps, 100)) if lam is None else lam
    dip = (tuple(src / H), (0.0, 0.0, 1.0), 1, f0 * ts, 1.0)
    t0 = time.perf_counter()
    oracle.tet_run((N, N, N), eps, oracle.SYMP4, dtn, steps, 1, [dip], [tuple(r / H) for r in recs])
    dt = time.perf_counter() - t0
    return n_edges(N) * steps / dt, dt


def _cpu_timed(code, threads=1, procs=1):
    """Runs `code` (python, prints the seconds of its timed part) in `procs`
    concurrent processes with OMP_NUM_THREADS=threads; returns the seconds of
    each.  A fresh process per sample, so the thread count takes effect."""
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    pre = f"import sys, time; sys.path.insert(0, {ROOT!r}); import numpy as np; import oracle\n"
    ps = [subprocess.Popen([sys.executable, "-c", pre + code], env=env, stdout=subprocess.PIPE, text=True) for _ in range(procs)]
    out = []
    for p in ps:
        o, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("CPU sample failed")
        out.append(float(o.strip().splitlines()[-1]))
    return out


def cpu_model():
    """The host CPU's model as /proc/cpuinfo or lscpu state it (Arm hosts
    list implementer and part numbers rather than a name)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for key in ("Model name:", "Vendor ID:"):
            for line in out.splitlines():
                if line.strip().startswith(key):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part", "hardware")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def cpu_rates(code, work, procs=None):
    """`work` units per run of `code`: single-core units/s, and the
    aggregate units/s of nproc concurrent single-threaded processes."""
    procs = procs or (os.cpu_count() or 1)
    one = _cpu_timed(code, 1, 1)[0]
    many = _cpu_timed(code, 1, procs)
    return {"single_core": work / one, "nproc_processes": procs * work / max(many), "processes": procs,
            "sample_s": one}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    steps = STEPS_PER_SOLVE   # per bench step: one full solve, about 5 s on 16 cores
    for _ in range(args.warmup):
        cpu_oracle_rate(5, threads)
    rates, secs = [], []
    for _ in range(args.steps):
        r, s = cpu_oracle_rate(steps, threads)
        rates.append(r)
        secs.append(s)
    value = float(np.mean(rates))
    sample = f"one full solve ({steps} time steps) per bench step (FP64 oracle, OpenMP)"
    print(json.dumps({
        "impl": "reference", "metric": "DOF-updates/s (32^3x6 tet Nedelec FEM, symp4, 2000 steps)", "value": value,
        "unit": "DOF-updates/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * float(np.mean(secs)) * STEPS_PER_SOLVE / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": "tet32_symp4_2000", "cells": N, "tets": 6 * N ** 3, "edges": n_edges(N),
                   "integrator": "symp4", "steps_per_solve": STEPS_PER_SOLVE, "parallelism": "replicas"},
        "cpu_baseline": {"value": value, "unit": "DOF-updates/s", "cores": threads, "kind": "port", "sample": sample,
                         "cpu_model": cpu_model()},
        "e2e": {"value": value, "unit": "DOF-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def fdtd64_sphere(steps=1000):
    """The FDTD family's FP64 workload at full size: 64^3 cells of 1 mm,
    vacuum with a centred sphere (radius 16 cells, eps_r 4), PEC, dt = 0.99
    x CFL, a Jz Ricker point source (10 GHz) at the centre, `steps` steps, Ez
    at 8 receivers on a 20-cell ring.  FP64 (bit-identical to the oracle and
    so to the reference, tests/test_fdtd_gpu.py) and FP32 device rates, and
    the FP64 oracle of the reference loop on the host cores."""
    import emsolvers_gb300 as ems
    n, h, eps0, mu0 = 64, 1e-3, 8.854187817e-12, 1.25663706212e-6
    dt = 0.99 * h / (C0 * np.sqrt(3))
    zz, yy, xx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    r = np.sqrt((xx + 0.5 - n / 2) ** 2 + (yy + 0.5 - n / 2) ** 2 + (zz + 0.5 - n / 2) ** 2)
    eps = np.where(r < 16, 4.0, 1.0) * eps0
    c = n // 2
    recs = [(c + int(round(20 * np.cos(a))), c + int(round(20 * np.sin(a))), c) for a in np.arange(8) * np.pi / 4]
    out = {"workload": "fdtd64_sphere_1000", "cells": n ** 3, "steps": steps, "receivers": len(recs)}
    for prec, name in ((ems.FP64, "fp64"), (ems.FP32, "fp32")):
        s = ems.FdtdSimulation((n, n, n), h, dt, eps0, mu0, 1, precision=prec)
        s.set_material(eps, np.zeros_like(eps))
        s.setSource_z((c, c, c), waveform=ems.WAVE_RICKER, f0=10e9)
        for q in recs:
            s.setObservationPoint(([], [], [q]))
        s.run(steps)
        s.run(steps)
        ms, _ = s.run_stats()
        out[f"cell_updates_per_s_{name}"] = n ** 3 * steps / (ms * 1e-3)
        out[f"ms_{name}"] = ms
        s.close()
    sample = 100
    code = (f"n={n}; h={h!r}; dt={dt!r}; eps0={eps0!r}; mu0={mu0!r}\n"
            "zz, yy, xx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing='ij')\n"
            "r = np.sqrt((xx + 0.5 - n / 2) ** 2 + (yy + 0.5 - n / 2) ** 2 + (zz + 0.5 - n / 2) ** 2)\n"
            "ids = (r < 16).astype(np.uint16)\n"
            "t0 = time.perf_counter()\n"
            f"oracle.fdtd_run(n, n, n, h, dt, eps0, mu0, 1, {sample}, [(2, (32, 32, 32), 1, 10e9, 1.0)], [([], [], [(52, 32, 32)])],"
            " material=(ids, np.array([eps0, 4 * eps0]), np.zeros(2)))\n"
            "print(time.perf_counter() - t0)\n")
    cpu = cpu_rates(code, n ** 3 * sample)
    out["cpu_baseline"] = {"value": cpu["single_core"], "unit": "cell-updates/s", "cores": 1, "kind": "port",
                           "nproc_processes_value": cpu["nproc_processes"], "processes": cpu["processes"],
                           "sample": f"{sample} steps of the same case, FP64 oracle of the reference loop "
                                     "(bit-identical to it); single core, and nproc concurrent single-threaded processes"}
    out["speedup_fp64_vs_cpu_core"] = out["cell_updates_per_s_fp64"] / cpu["single_core"]
    return out


def tet32_symp2(steps=STEPS_PER_SOLVE):
    """The headline mesh and material with the second-order symplectic
    (leapfrog, symplectic_2) step instead of the fourth-order one: FP32
    device rate and the FP32-vs-FP64 trace error over the whole run."""
    import emsolvers_gb300 as ems
    eps, f0, src, recs = workload()
    out = {"workload": "tet32_symp2_2000", "steps": steps, "integrator": "symp2"}
    tr = {}
    for prec, name in ((ems.FP32, "fp32"), (ems.FP64, "fp64")):
        sim = ems.TetFemSimulation((N, N, N), H, 1, ems.SYMP2, prec, dt=0.0, cfl_fraction=0.9)
        sim.set_material(eps)
        sim.add_dipole(src, (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0, 1.0)
        for r in recs:
            sim.add_receiver(r)
        sim.run(steps)
        sim.reset()
        sim.run(steps)
        ms, _ = sim.run_stats()
        out[f"dof_updates_per_s_{name}"] = n_edges(N) * steps / (ms * 1e-3)
        out["dt_s"] = sim.time_step()[0]
        tr[name] = sim.traces()[..., 1:]
        sim.close()
    out["fp32_vs_fp64_trace_rel_l2"] = float(np.linalg.norm(tr["fp32"] - tr["fp64"]) / np.linalg.norm(tr["fp64"]))
    return out


def fdtd_512(steps=4000, n=512, nrec=64, compare_fp64=True):
    """n^3 (512^3) Yee FDTD with a 10-cell CPML: eps_r log-uniform [1, 10] on
    16^3-cell blocks, sigma U[0, 0.05] S/m, 4 Ricker point sources (f0 U[5,
    15] GHz) at random interior cells, `steps` steps, `nrec` receivers (Ex,
    Ey, Ez at one cell each).  FP32 device rate, the step's bytes against HBM
    and the E kernel alone; with compare_fp64 the same run in FP64 and the
    FP32-vs-FP64 trace error over all receivers and steps."""
    import emsolvers_gb300 as ems
    h = 1e-3
    eps0, mu0 = 8.854187817e-12, 1.25663706212e-6
    dt = 0.99 * h / (C0 * np.sqrt(3))
    rng = np.random.default_rng(SEED)
    nb = n // 16
    blk_eps = 10 ** rng.uniform(0, 1, nb ** 3) * eps0
    blk_sig = rng.uniform(0, 0.05, nb ** 3)
    idx = (np.arange(n) // 16)
    cell_blk = (idx[None, None, :] + nb * (idx[None, :, None] + nb * idx[:, None, None])).reshape(-1)
    srcs = [(tuple(int(v) for v in rng.integers(20, n - 20, 3)), float(rng.uniform(5e9, 15e9))) for _ in range(4)]
    recs = [tuple(int(v) for v in rng.integers(12, n - 12, 3)) for _ in range(nrec)]

    def one(precision):
        s = ems.FdtdSimulation((n, n, n), h, dt, eps0, mu0, 1, precision=precision, pml_cells=10, pml_order=3.0,
                               pml_kappa_max=1.0, pml_alpha_max=0.0, pml_reflection=1e-6)
        s.set_material(blk_eps[cell_blk], blk_sig[cell_blk])
        for c, f in srcs:
            s.setSource_z(c, waveform=ems.WAVE_RICKER, f0=f)
        for r in recs:
            s.setObservationPoint(([r], [r], [r]))
        s.run(40)          # warm-up; the handle's first run of >= 40 steps picks the launch shape
        s.reset()
        s.run(steps)
        ms, launches = s.run_stats()
        return s, ms, launches

    s, ms, launches = one(ems.FP32)
    kms, kbytes, kname = s.time_dominant_kernel(10)
    shape = s.launch_shape()
    tr32 = s.traces()
    s.close()
    cells = n ** 3
    npml = cells - (n - 20) ** 3
    # one step's algorithmic bytes: E and H read and written (12 words per
    # cell), the 2-byte material id per cell, 12 CPML psi values read and
    # written per cell inside the slabs
    step_bytes = 4.0 * 12 * cells + 2.0 * cells + 4.0 * 24 * npml
    out = {"workload": f"fdtd{n}_fp32_cpml10_{steps}", "steps": steps, "receivers": nrec, "sources": len(srcs),
           "ms_per_step": ms / steps, "launches": int(launches), "launch_shape": list(shape[:2]),
           "cell_updates_per_s": cells * steps / (ms * 1e-3), "dof_updates_per_s": 6 * cells * steps / (ms * 1e-3),
           "step_bytes": step_bytes, "step_gbs": step_bytes / (ms / steps * 1e-3) / 1e9,
           "kernel": kname, "kernel_ms": kms, "kernel_bytes": kbytes, "kernel_gbs": kbytes / (kms * 1e-3) / 1e9}
    if compare_fp64:
        s, ms64, _ = one(ems.FP64)
        tr64 = s.traces()
        s.close()
        out["fp64_ms_per_step"] = ms64 / steps
        out["fp32_vs_fp64_trace_rel_l2"] = float(np.linalg.norm(tr32 - tr64) / np.linalg.norm(tr64))
    return out


def head_solve(steps=STEPS_PER_SOLVE):
    """One headline solve (setup, then `steps` time steps) for profiling."""
    import emsolvers_gb300 as ems
    eps, f0, src, recs = workload()
    sim = ems.TetFemSimulation((N, N, N), H, 1, ems.SYMP4, ems.FP32, dt=0.0, cfl_fraction=0.9, time_frequency=1)
    sim.set_material(eps)
    sim.add_dipole(src, (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0, 1.0)
    for r in recs:
        sim.add_receiver(r)
    sim.run(steps)
    ms, launches = sim.run_stats()
    sim.close()
    return {"workload": "tet32_symp4", "steps": steps, "device_ms": ms, "launches": launches,
            "dof_updates_per_s": n_edges(N) * steps / (ms * 1e-3)}


def batch64(nshots=64, steps=3000, sample=8, sample_steps=300, o2_steps=300, o2_sample=2, o2_sample_steps=50):
    """Batched forward shots: nshots cubes of side n ~ U[12,40] (6 n^3
    tetrahedra each), first- or second-order Nedelec by coin flip, eps_r ~
    U[1,6] per tet, one Ricker dipole each, 4th-order symplectic, `steps`
    steps, FP32, one common time step (the stiffest shot's).  The shots of
    each order advance together in one batch handle (all shots of the order
    in every launch, the time loop in CUDA graphs); the two handles run back
    to back.  The order-1 batch runs all `steps`; the order-2 batch runs
    `o2_steps` of them (its rate scaled to `steps`).  Compared with the
    plain per-shot FP64 GPU path on `sample` order-1 and `o2_sample` order-2
    shots (same time step, sample steps scaled to `steps`)."""
    import emsolvers_gb300 as ems
    rng = np.random.default_rng(SEED + 4)
    sides = rng.integers(12, 41, nshots)
    cells = [(int(n), int(n), int(n)) for n in sides]
    eps = [rng.uniform(1.0, 6.0, 6 * n ** 3) for n in sides]
    pos = [np.array([n, n, n]) * rng.uniform(0.3, 0.7, 3) * H for n in sides]
    rec = [np.array([n, n, n]) * rng.uniform(0.2, 0.8, 3) * H for n in sides]
    orders = rng.integers(1, 3, nshots)
    f0 = C0 / (10 * H * np.sqrt(3.5))
    groups = {o: [s for s in range(nshots) if orders[s] == o] for o in (1, 2)}

    def handle(o, dt):
        sh = groups[o]
        b = ems.TetFemBatch([cells[s] for s in sh], H, order=o, integrator=ems.SYMP4, precision=ems.FP32, dt=dt,
                            cfl_fraction=0.9)
        b.set_material(np.concatenate([eps[s] for s in sh]))
        for k, s in enumerate(sh):
            b.add_dipole(k, pos[s], (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0)
            b.add_receiver(k, rec[s])
        return b

    dts = []
    for o in (1, 2):
        if groups[o]:
            b = handle(o, 0.0)
            dts.append(b.time_step()[0])
            b.close()
    dt = min(dts)
    res = {}
    for o in (1, 2):
        if not groups[o]:
            continue
        b = handle(o, dt)
        nst = steps if o == 1 else min(o2_steps, steps)
        b.run(20)
        b.reset()
        b.run(nst)
        ms, launches = b.run_stats()
        kms, kbytes, kname = b.time_dominant_kernel(20)
        res[o] = {"shots": len(groups[o]), "ms": ms * steps / nst, "run_steps": nst, "launches_per_step": launches / nst,
                  "kernel": kname, "kernel_us": kms * 1e3, "kernel_gbs": kbytes / (kms * 1e-3) / 1e9,
                  "launch_shape": list(b.launch_shape()),
                  "dofs": int(sum(n_edges(int(sides[s])) if o == 1 else n_dofs2(int(sides[s])) for s in groups[o]))}
        b.close()
    ms_batch = sum(r["ms"] for r in res.values())
    # plain per-shot paths on a sample of each order
    per = {ems.FP64: 0.0, ems.FP32: 0.0}
    picks = {}
    for o, k, st in ((1, sample, sample_steps), (2, o2_sample, o2_sample_steps)):
        if not groups[o]:
            continue
        pick = rng.choice(groups[o], size=min(k, len(groups[o])), replace=False)
        picks[o] = (len(pick), st)
        for prec in (ems.FP64, ems.FP32):
            t = []
            for s in pick:
                one = ems.TetFemSimulation(cells[s], H, o, ems.SYMP4, prec, dt=dt)
                one.set_material(eps[s])
                one.add_dipole(pos[s], (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0)
                one.add_receiver(rec[s])
                one.run(3)
                one.reset()
                one.run(st)
                t.append(one.run_stats()[0] * steps / st)
                one.close()
            per[prec] += np.mean(t) * len(groups[o])   # the order's shots at the sample's mean time
    shots_batch = nshots / (ms_batch * 1e-3)
    shots_fp64 = nshots / (per[ems.FP64] * 1e-3)
    shots_fp32 = nshots / (per[ems.FP32] * 1e-3)
    dofs = sum(r["dofs"] for r in res.values())
    # CPU: one order-1 shot of the batch's mean size, FP64 oracle, sample steps scaled
    nm = int(round(np.cbrt(np.mean(sides.astype(float) ** 3))))
    cpu_steps = 100
    code = (f"n = {nm}; eps = np.random.default_rng(0).uniform(1.0, 6.0, 6 * n ** 3)\n"
            f"dip = ((0.5 * n, 0.47 * n, 0.52 * n), (0.0, 0.0, 1.0), 1, {f0 * H / C0!r}, 1.0)\n"
            f"dtn = {dt * C0 / H!r}\n"
            "t0 = time.perf_counter()\n"
            f"oracle.tet_run((n, n, n), eps, oracle.SYMP4, dtn, {cpu_steps}, 1, [dip], [(0.3 * n, 0.6 * n, 0.4 * n)])\n"
            "print(time.perf_counter() - t0)\n")
    cpu = cpu_rates(code, cpu_steps / steps)
    return {"workload": "tet_batch64_symp4_3000_mixed_order", "shots": nshots, "steps": steps,
            "tets": int(sum(6 * sides ** 3)), "order_1_shots": len(groups[1]), "order_2_shots": len(groups[2]),
            "dofs": int(dofs), "dt_s": dt, "batch_ms": ms_batch,
            "per_order": {str(o): r for o, r in res.items()},
            "order_2_timing": f"order-2 batch timed over {min(o2_steps, steps)} of the {steps} steps, scaled",
            "shots_per_s_fp32_batched": shots_batch, "shots_per_s_fp64_per_shot": shots_fp64,
            "shots_per_s_fp32_per_shot": shots_fp32, "speedup_vs_fp64_per_shot": shots_batch / shots_fp64,
            "dof_updates_per_s": dofs * steps / (ms_batch * 1e-3),
            "per_shot_sample": "; ".join(f"order {o}: {n} shots x {st} steps, scaled to {steps}" for o, (n, st) in picks.items()),
            "cpu_baseline": {"value": cpu["single_core"], "unit": "shots/s (order 1)", "cores": 1, "kind": "port",
                             "nproc_processes_value": cpu["nproc_processes"], "processes": cpu["processes"],
                             "sample": f"one order-1 {nm}^3 x 6 tet shot (the batch's mean size), {cpu_steps} steps of the "
                                       f"FP64 oracle scaled to {steps}; single core, and nproc concurrent single-threaded "
                                       "processes"}}


def hex72(steps=200, order=2, sample_steps=10):
    """The reference's own solver family: symplectic_4, OFEM order 2 on a
    72^3 fine grid (1,151,064 edge DOFs; the element size and time step of
    the symplectic_4 order-2 golden case), FP64 (bit-identical to the
    reference) and FP32 device rates, against the FP64 oracle port of the
    reference's loop on the host cores (`sample_steps` steps)."""
    import emsolvers_gb300 as ems
    import oracle
    g = 72
    h, dt, eps0, mu0 = 0.1, 9.629166007732144e-11, 8.8541878128e-12, 1.25663706212e-06
    kdir = os.path.join(ROOT, "tests", "golden", "kmat")
    dofs = 3 * g * (g + 1) ** 2
    out = {"workload": f"hex{g}_symp4_o{order}_ofem", "dofs": dofs, "steps": steps, "order": order}
    for prec, name in ((ems.FP64, "fp64"), (ems.FP32, "fp32")):
        s = ems.HexFemSimulation(order, (g, g, g), h, dt, eps0, mu0, 2, 1, integrator=ems.SYMP4, precision=prec,
                                 kmat_dir=kdir)
        s.setSource_z((g // 2, g // 2, g // 2))
        s.setObservationPoint((g // 2 + 6, g // 2 - 4, g // 2 + 2))
        s.run(5)
        s.reset()
        s.run(steps)
        ms, _ = s.run_stats()
        out[f"dof_updates_per_s_{name}"] = dofs * steps / (ms * 1e-3)
        s.close()
    kmat = oracle.load_kmat(os.path.join(kdir, f"{order}.csv"))
    t0 = time.perf_counter()
    oracle.hexfem_run(order, (g, g, g), h, dt, eps0, mu0, 2, oracle.SYMP4, kmat, sample_steps,
                      sources=[(2, (g // 2, g // 2, g // 2))], observations=[(g // 2 + 6, g // 2 - 4, g // 2 + 2)])
    cpu = dofs * sample_steps / (time.perf_counter() - t0)
    out["cpu_baseline"] = {"value": cpu, "unit": "DOF-updates/s", "cores": 1, "kind": "port",
                           "sample": f"{sample_steps} steps, FP64 oracle of the reference loop (bit-identical to it, "
                                     "serial like the reference built without nvc++)"}
    out["speedup_fp64_vs_cpu"] = out["dof_updates_per_s_fp64"] / cpu
    return out


def tet2_forward(n=48, steps=200):
    """Second-order (20-DOF) tetrahedra on an n^3 x 6 tet cube (the blob model
    of the inversion configuration), one Ricker dipole, 8 receivers, symp4:
    FP32 and FP64 device rates over `steps` steps, and one Chebyshev mass
    iteration (element pass + entity pass) timed alone."""
    import emsolvers_gb300 as ems
    rng = np.random.default_rng(SEED + 7)
    eps = blob_model(n, rng)
    f0 = C0 / (10 * H * np.sqrt(2.0))
    src = np.array([0.5, 0.47, 0.52]) * n * H
    recs = [rng.uniform(0.1, 0.9, 3) * n * H for _ in range(8)]
    out = {"workload": f"tet{n}_order2_symp4", "order": 2, "dofs": n_dofs2(n), "tets": 6 * n ** 3, "steps": steps}
    dt = None
    for prec, name in ((ems.FP32, "fp32"), (ems.FP64, "fp64")):
        s = ems.TetFemSimulation((n, n, n), H, 2, ems.SYMP4, prec, dt=dt or 0.0, cfl_fraction=0.9)
        s.set_material(eps)
        s.add_dipole(src, (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0, 1.0)
        for r in recs:
            s.add_receiver(r)
        dt = dt or s.time_step()[0]
        s.run(3)
        s.reset()
        s.run(steps)
        ms, launches = s.run_stats()
        out[f"dof_updates_per_s_{name}"] = n_dofs2(n) * steps / (ms * 1e-3)
        out[f"ms_per_step_{name}"] = ms / steps
        out[f"launches_per_step_{name}"] = launches / steps
        kms, kbytes, kname = s.time_dominant_kernel(20)
        out[f"cheb_iteration_us_{name}"] = kms * 1e3
        out[f"cheb_iteration_gbs_{name}"] = kbytes / (kms * 1e-3) / 1e9
        s.close()
    out["dt_s"] = dt
    out["fp32_speedup_vs_fp64"] = out["dof_updates_per_s_fp32"] / out["dof_updates_per_s_fp64"]
    # CPU: the FP64 oracle of the same scheme on the 16^3 model of the recipe,
    # `cpu_steps` steps, DOF-updates/s
    nc, cpu_steps = min(n, 16), 2
    code = (f"import bench\n"
            f"n = {nc}; eps = bench.blob_model(n, np.random.default_rng({SEED + 7}))\n"
            f"dip = ((0.5 * n, 0.47 * n, 0.52 * n), (0.0, 0.0, 1.0), 1, {f0 * H / C0!r}, 1.0)\n"
            f"dtn = {dt * C0 / H!r}\n"
            "t0 = time.perf_counter()\n"
            f"oracle.tet2_run((n, n, n), eps, oracle.SYMP4, dtn, {cpu_steps}, 1, [dip], [(0.3 * n, 0.6 * n, 0.4 * n)])\n"
            "print(time.perf_counter() - t0)\n")
    cpu = cpu_rates(code, n_dofs2(nc) * cpu_steps)
    out["cpu_baseline"] = {"value": cpu["single_core"], "unit": "DOF-updates/s", "cores": 1, "kind": "port",
                           "nproc_processes_value": cpu["nproc_processes"], "processes": cpu["processes"],
                           "sample": f"{nc}^3 x 6 tets of the same recipe, {cpu_steps} steps of the FP64 oracle (setup "
                                     "included); single core, and nproc concurrent single-threaded processes"}
    return out


def blob_model(n, rng, background=2.0, nblob=3):
    """Per-tet eps_r: background plus nblob Gaussian blobs (amplitude U[1,3],
    width U[4,8] cells) evaluated at the tetrahedron centroids."""
    # centroid of Kuhn tetrahedron p of cell (i,j,k): cell corner + (3/4, 2/4, 1/4) along its axis order
    perm = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    off = np.zeros((6, 3))
    for p, (a, b, c) in enumerate(perm):
        off[p, a], off[p, b], off[p, c] = 0.75, 0.5, 0.25
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    corner = np.stack([i.ravel(), j.ravel(), k.ravel()], 1).astype(float)
    cen = (corner[:, None, :] + off[None, :, :]).reshape(-1, 3)
    eps = np.full(cen.shape[0], background)
    for _ in range(nblob):
        c = rng.uniform(0.25, 0.75, 3) * n
        amp, width = rng.uniform(1.0, 3.0), rng.uniform(4.0, 8.0)
        eps += amp * np.exp(-np.sum((cen - c) ** 2, 1) / (2 * width ** 2))
    return eps


def adjoint16(n=48, nshots=16, nrec=32, steps=4000, nsnap=64, fd_elements=32, fd_h=1e-4, cpu_steps=20, order=1,
              full_steps=4000, fd_n=None, tf_backward=True):
    """Forward + adjoint misfit gradient: nshots Ricker dipole shots on an
    n^3 x 6 tet cube (true eps_r = 2 + 3 Gaussian blobs, start model 2), nrec
    receivers per shot, symp4, `steps` steps, nsnap snapshots; L2 and TF
    envelope misfits.  FP32 batched (all shots in one handle) against the
    plain per-shot FP64 GPU path (shot 0, the whole run).  Checks: FP32 vs
    FP64 traces and gradient over the whole run of shot 0, and central
    differences (relative step fd_h, FP64, all perturbed models in one
    batch) of the L2 misfit on fd_elements random tetrahedra.  With steps <
    full_steps the run is a sample of the full-length run: rates are scaled
    by steps / full_steps and the accuracy figures cover the sample.
    fd_n: run the central differences on an fd_n^3 model of the same recipe
    instead (same sources and receivers in relative position), where FP64
    runs are cheap; tf_backward=False reports the TF envelope misfit
    without its backward sweep."""
    import emsolvers_gb300 as ems
    rng = np.random.default_rng(SEED + 5)
    true = blob_model(n, rng)
    start = np.full(true.size, 2.0)
    f0 = C0 / (10 * H * np.sqrt(2.0))
    src = [rng.uniform(0.2, 0.8, 3) * n * H for _ in range(nshots)]
    rec = [rng.uniform(0.1, 0.9, 3) * n * H for _ in range(nrec)]
    probe = ems.TetFemSimulation((n, n, n), H, order, ems.SYMP4, ems.FP32, dt=0.0, cfl_fraction=0.9)
    probe.set_material(start)
    dt, _ = probe.time_step()
    probe.close()

    def handle(precision, shots, model, nn=n):
        sc = nn / n   # sources and receivers keep their relative positions
        b = ems.TetFemBatch([(nn, nn, nn)] * len(shots), H, order=order, integrator=ems.SYMP4, precision=precision, dt=dt)
        b.set_material(np.tile(model, len(shots)) if np.ndim(model) == 1 and len(model) == 6 * nn ** 3 else model)
        for k, sh in enumerate(shots):
            b.add_dipole(k, src[sh] * sc, (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0)
            for r in rec:
                b.add_receiver(k, r * sc)
        return b

    shots = list(range(nshots))
    b = handle(ems.FP32, shots, true)
    b.run(steps)
    obs = b.traces()
    b.close()
    import torch
    torch.cuda.synchronize()
    b = handle(ems.FP32, shots, start)
    t0 = time.perf_counter()
    b.set_material(np.tile(start, nshots))
    b.set_checkpoints(nsnap)
    b.time_step()
    ts = [time.perf_counter()]
    b.reset()
    b.run(steps)
    ts.append(time.perf_counter())
    fwd_ms, _ = b.run_stats()
    J, tg = ems.trace_misfit(b.traces(), obs, ems.MISFIT_L2)
    ts.append(time.perf_counter())
    g32 = b.backward(tg).reshape(nshots, -1)
    ts.append(time.perf_counter())
    wall32 = ts[-1] - t0
    stages = {"setup_s": ts[0] - t0, "forward_s": ts[1] - ts[0], "misfit_s": ts[2] - ts[1], "backward_s": ts[3] - ts[2]}
    # the TF envelope misfit on the same recorded run (a second backward sweep)
    t1 = time.perf_counter()
    Jtf, gtf = None, None
    if tf_backward:
        Jtf, tgtf = ems.trace_misfit(b.traces(), obs, ems.MISFIT_TF_ENVELOPE)
        gtf = b.backward(tgtf).reshape(nshots, -1).sum(0)
    tf_s = time.perf_counter() - t1
    tr32_0 = b.traces()[:nrec]
    b.close()
    # plain per-shot FP64 GPU path: shot 0, the whole run
    one = handle(ems.FP64, [0], start)
    one.set_checkpoints(nsnap)
    obs0 = obs[:nrec]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    one.set_material(start)
    one.time_step()
    one.reset()
    one.run(steps)
    J0, tg0 = ems.trace_misfit(one.traces(), obs0, ems.MISFIT_L2)
    g64_0 = one.backward(tg0)
    wall64 = time.perf_counter() - t0
    tr64 = one.traces()
    one.close()
    tr_err = float(np.linalg.norm(tr32_0[..., 1:] - tr64[..., 1:]) / np.linalg.norm(tr64[..., 1:]))
    g_err = float(np.linalg.norm(g32[0] - g64_0) / np.linalg.norm(g64_0))
    # central differences of J0 on fd_elements tetrahedra, FP64, one batch of
    # 2 fd_elements perturbed copies of the start model (shot 0 each)
    t1 = time.perf_counter()
    nf, start_f, obs_f, g_ref = n, start, obs0, g64_0
    if fd_n:   # the same check on the small model: its own observed traces and FP64 adjoint
        nf = fd_n
        true_f = blob_model(nf, np.random.default_rng(SEED + 6))
        start_f = np.full(true_f.size, 2.0)
        h = handle(ems.FP64, [0], true_f, nf)
        h.run(steps)
        obs_f = h.traces()
        h.close()
        h = handle(ems.FP64, [0], start_f, nf)
        h.set_checkpoints(nsnap)
        h.reset()
        h.run(steps)
        g_ref = h.backward(ems.trace_misfit(h.traces(), obs_f, ems.MISFIT_L2)[1])
        h.close()
    pick = rng.choice(start_f.size, size=fd_elements, replace=False)
    models = np.tile(start_f, 2 * fd_elements).reshape(2 * fd_elements, -1)
    for q, t in enumerate(pick):
        models[2 * q, t] += fd_h * start_f[t]
        models[2 * q + 1, t] -= fd_h * start_f[t]
    fd = handle(ems.FP64, [0] * (2 * fd_elements), models.reshape(-1), nf)
    fd.run(steps)
    trs = fd.traces().reshape(2 * fd_elements, nrec, -1, 4)
    fd.close()
    fd_s = time.perf_counter() - t1
    Jp = np.array([ems.trace_misfit(trs[k], obs_f, ems.MISFIT_L2)[0] for k in range(2 * fd_elements)])
    g_fd = (Jp[0::2] - Jp[1::2]) / (2 * fd_h * start_f[pick])
    fd_err = float(np.linalg.norm(g_ref[pick] - g_fd) / np.linalg.norm(g_fd))
    scale = steps / full_steps   # rates of the full-length run from a step sample
    cpu = None
    # CPU: the FP64 oracle adjoint of one shot over cpu_steps steps, scaled
    code = (f"n = {n}; rng = np.random.default_rng(0); eps = np.full(6 * n ** 3, 2.0)\n"
            f"dip = ({tuple(src[0] / H)!r}, (0.0, 0.0, 1.0), 1, {f0 * H / C0!r}, 1.0)\n"
            f"recs = {[tuple(r / H) for r in rec]!r}\n"
            f"dtn = {dt * C0 / H!r}\n"
            f"tr, _, _ = oracle.tet_run((n, n, n), eps, oracle.SYMP4, dtn, {cpu_steps}, 1, [dip], recs)\n"
            "t0 = time.perf_counter()\n"
            f"tr, _, _ = oracle.tet_run((n, n, n), eps, oracle.SYMP4, dtn, {cpu_steps}, 1, [dip], recs)\n"
            "g = tr.copy(); g[..., 0] = 0.0\n"
            f"oracle.tet_gradient((n, n, n), eps, oracle.SYMP4, dtn, {cpu_steps}, g, 1, [dip], recs)\n"
            "print(time.perf_counter() - t0)\n")
    if order == 1 and cpu_steps > 0:
        cpu = cpu_rates(code, cpu_steps / full_steps)   # shots per run of the sample
    out = {"workload": f"tet{n}_adjoint_{nshots}shots_symp4_{full_steps}" + ("" if order == 1 else "_order2"),
           "tets_per_shot": int(true.size),
            "shots": nshots, "receivers_per_shot": nrec, "steps": steps, "snapshots": nsnap,
            "misfits": ["L2", "TF_envelope"] if tf_backward else ["L2"],
            "order": order, "dt_s": dt, "misfit_l2": J, "misfit_tf_envelope": Jtf,
            "grad_norm_l2": float(np.linalg.norm(g32.sum(0))),
            "grad_norm_tf": float(np.linalg.norm(gtf)) if gtf is not None else None,
            "fp32_batched_s": wall32, "fp32_forward_ms": fwd_ms, "fp32_stages": stages, "tf_envelope_backward_s": tf_s,
            "shots_per_s_fp32_batched": nshots / wall32 * scale, "shots_per_s_fp64_per_shot": 1.0 / wall64 * scale,
            "speedup_vs_fp64_per_shot": (nshots / wall32) * wall64,
            "fp64_per_shot": "shot 0, the whole run: material upload, FP64 mass setup, recorded forward, misfit, backward",
            "fp32_vs_fp64_trace_rel_l2": tr_err, "fp32_vs_fp64_grad_rel_l2": g_err,
            "fp32_vs_fp64_over": f"shot 0, all {steps} steps (forward traces and gradient)",
            "fd_check": {"elements": fd_elements, "h_rel": fd_h, "fp64_adjoint_vs_central_diff_rel_l2": fd_err,
                         "seconds": fd_s, "model": f"{nf}^3 x 6 tets, shot 0, {steps} steps"},
            "timing": "wall clock: material upload + FP64 mass setup + recorded forward + misfit + backward"}
    if steps < full_steps:
        out["step_sample"] = (f"{steps} of the {full_steps} steps ({nsnap} snapshots), all {nshots} shots; shots/s "
                              f"scaled to the full run, accuracy figures over the sample")
    if cpu is not None:
        out["cpu_baseline"] = {"value": cpu["single_core"], "unit": "shots/s", "cores": 1, "kind": "port",
                               "nproc_processes_value": cpu["nproc_processes"], "processes": cpu["processes"],
                               "sample": f"one shot, {cpu_steps} steps forward + adjoint (FP64 oracle), scaled to "
                                         f"{full_steps}; single core, and nproc concurrent single-threaded processes"}
    return out


def run_gpu(args):
    import torch
    import emsolvers_gb300 as ems

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    eps, f0, src, recs = workload()
    ts = H / C0
    sim = ems.TetFemSimulation((N, N, N), H, 1, ems.SYMP4, ems.FP32, dt=0.0, cfl_fraction=0.9, time_frequency=1)
    sim.set_material(eps)
    sim.add_dipole(src, (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0, 1.0)
    for r in recs:
        sim.add_receiver(r)
    dt, lim = sim.time_step()
    l2 = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(max(args.warmup, 3)):
        sim.reset()
        sim.run(STEPS_PER_SOLVE)
    # ---- device-resident timing: K solves, L2 flushed between them
    clocks = Clocks()
    dev_ms, launches = [], 0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        sim.reset()
        flush_l2(l2)
        torch.cuda.synchronize()
        sim.run(STEPS_PER_SOLVE)
        ms, nl = sim.run_stats()
        dev_ms.append(ms)
        launches += nl
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    total_ms = float(np.sum(dev_ms))
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    dofs = n_edges(N)
    value = world * dofs * STEPS_PER_SOLVE * args.steps / (total_ms * 1e-3)
    traces = sim.traces()
    # ---- end to end through the C ABI from host buffers
    e2e_ms = []
    for _ in range(args.steps):
        flush_l2(l2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.set_material(eps)          # host -> device, FP64 mass setup + stability limit
        sim.reset()
        sim.run(STEPS_PER_SOLVE)
        tr = sim.traces()              # device -> host
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e = world * dofs * STEPS_PER_SOLVE * args.steps / (np.sum(e2e_ms) * 1e-3)
    # ---- dominant kernel roofline.  In the loop every substep is one launch
    # of the fused step (3 per symp4 step, replayed from CUDA graphs); the
    # solve's device time over those launches is the in-loop time per launch
    # (an upper bound: it also holds the two half drifts and the graph launch
    # gaps).  The same kernel timed alone by repeated launches outside a graph
    # is reported beside it.
    kms, kbytes, kname = sim.time_dominant_kernel(200)
    block = list(sim.launch_shape())
    peak, peak_kind = peaks()
    step_launches = 3 * STEPS_PER_SOLVE
    inloop_ms = float(np.mean(dev_ms)) / step_launches
    achieved = kbytes / (inloop_ms * 1e-3) / 1e9
    out = {
        "metric": "DOF-updates/s (32^3x6 tet Nedelec FEM, symp4, 2000 steps)", "value": value, "unit": "DOF-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded eps_r U[1,4] per tet)",
        "config": {"workload": "tet32_symp4_2000", "cells": N, "tets": 6 * N ** 3, "edges": dofs, "integrator": "symp4",
                   "steps_per_solve": STEPS_PER_SOLVE, "dt_s": dt, "dt_limit_s": lim, "receivers": len(recs),
                   "l2": "flushed between solves (512 MB write)", "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": float(e2e), "unit": "DOF-updates/s", "h2d_bytes_per_step": int(eps.nbytes),
                "d2h_bytes_per_step": int(tr.nbytes)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     # DRAM bytes of one step launch from the ncu capture in
                     # profiles/tet_slot_tet32_symp4.md (cold fill: the 7.1 MB
                     # working set is L2-resident in the timed loop)
                     "traffic": TRAFFIC_PER_LAUNCH, "kernel": kname, "kernel_us": inloop_ms * 1e3,
                     "kernel_us_alone": kms * 1e3, "launches_per_solve": step_launches, "bytes_per_launch": kbytes,
                     "timing": "in-loop: solve device time / fused-step launches (includes the half drifts and launch gaps)",
                     "launch_shape": block, "peak_source": peak_kind},
        "clocks": clk,
        "wall_s": wall,
    }
    if rank == 0:
        if not args.no_cpu:
            secs = [cpu_oracle_rate(STEPS_PER_SOLVE, os.cpu_count() or 1)[1] for _ in range(3)]
            r = n_edges(N) * 3 * STEPS_PER_SOLVE / sum(secs)
            sample = 200
            code = ("import bench\n"
                    "eps, f0, src, recs = bench.workload()\n"
                    f"dtn = {dt * C0 / H!r}\n"
                    "dip = (tuple(src / bench.H), (0.0, 0.0, 1.0), 1, f0 * bench.H / bench.C0, 1.0)\n"
                    "t0 = time.perf_counter()\n"
                    f"oracle.tet_run((bench.N,) * 3, eps, oracle.SYMP4, dtn, {sample}, 1, [dip], [tuple(q / bench.H) for q in recs])\n"
                    "print(time.perf_counter() - t0)\n")
            per = cpu_rates(code, n_edges(N) * sample)
            out["cpu_baseline"] = {"value": r, "unit": "DOF-updates/s", "cores": os.cpu_count() or 1, "kind": "port",
                                   "cpu_model": cpu_model(),
                                   "sample": f"three full solves ({STEPS_PER_SOLVE} time steps each), FP64 oracle, "
                                             f"{sum(secs):.1f} s",
                                   "single_core_value": per["single_core"], "nproc_processes_value": per["nproc_processes"],
                                   "processes": per["processes"],
                                   "per_core_sample": f"{sample} steps in one thread, and in nproc concurrent single-threaded "
                                                      "processes (one solve each)"}
        if not args.no_fdtd:
            try:
                out["fdtd64_sphere"] = fdtd64_sphere()
            except Exception as e:  # secondary measurement only
                out["fdtd64_sphere"] = {"error": str(e)}
        if not args.no_batch:
            try:
                out["tet32_symp2"] = tet32_symp2()
            except Exception as e:  # secondary measurement only
                out["tet32_symp2"] = {"error": str(e)}
        if not args.no_batch:
            try:
                out["batch64"] = batch64()
            except Exception as e:  # secondary measurement only
                out["batch64"] = {"error": str(e)}
        if not args.no_hex:
            try:
                out["hex72"] = hex72()
            except Exception as e:  # secondary measurement only
                out["hex72"] = {"error": str(e)}
        if not args.no_adjoint:
            try:
                out["tet48_order2"] = tet2_forward(n=48, steps=100)
            except Exception as e:  # secondary measurement only
                out["tet48_order2"] = {"error": str(e)}
            try:
                out["adjoint16_order2"] = adjoint16(order=2, nshots=2, steps=200, nsnap=4, fd_elements=8, fd_n=12,
                                                    tf_backward=False)
            except Exception as e:  # secondary measurement only
                out["adjoint16_order2"] = {"error": str(e)}
            try:
                out["adjoint16"] = adjoint16()
            except Exception as e:  # secondary measurement only
                out["adjoint16"] = {"error": str(e)}
        if not args.no_fdtd:
            try:
                out["fdtd_512"] = fdtd_512()
                out["fdtd_512"]["hbm_frac"] = out["fdtd_512"]["kernel_gbs"] / peak
                out["fdtd_512"]["step_hbm_frac"] = out["fdtd_512"]["step_gbs"] / peak
            except Exception as e:  # secondary measurement only
                out["fdtd_512"] = {"error": str(e)}
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fdtd", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-hex", action="store_true")
    ap.add_argument("--only", choices=["head", "batch", "fdtd", "adjoint", "hex", "sphere", "symp2", "tet2"],
                    help="run one secondary workload alone and print its JSON (for profiling)")
    ap.add_argument("--fdtd-n", type=int, default=512, help="FDTD cube side for --only fdtd")
    ap.add_argument("--head-steps", type=int, default=STEPS_PER_SOLVE, help="time steps for --only head")
    ap.add_argument("--batch-steps", type=int, default=3000, help="time steps for --only batch")
    ap.add_argument("--batch-sample", type=int, default=8, help="per-shot FP64 sample size for --only batch")
    ap.add_argument("--adj-n", type=int, default=48, help="cube side for --only adjoint")
    ap.add_argument("--adj-steps", type=int, default=4000, help="time steps for --only adjoint")
    ap.add_argument("--adj-shots", type=int, default=16, help="shots for --only adjoint")
    ap.add_argument("--adj-fd", type=int, default=32, help="central-difference elements for --only adjoint")
    ap.add_argument("--adj-order", type=int, default=1, choices=[1, 2], help="Nedelec order for --only adjoint")
    ap.add_argument("--adj-fd-n", type=int, default=0, help="cube side of the central-difference model (0: the same)")
    ap.add_argument("--adj-no-tf", action="store_true", help="skip the TF envelope backward sweep")
    ap.add_argument("--fdtd-steps", type=int, default=4000, help="time steps for --only fdtd")
    ap.add_argument("--tet2-steps", type=int, default=200, help="time steps for --only tet2")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        fn = {"head": lambda: head_solve(args.head_steps),
              "batch": lambda: batch64(steps=args.batch_steps, sample=args.batch_sample,
                                       sample_steps=min(300, args.batch_steps)),
              "fdtd": lambda: fdtd_512(n=args.fdtd_n, steps=args.fdtd_steps, compare_fp64=args.fdtd_steps >= 1000),
              "hex": hex72, "sphere": fdtd64_sphere, "symp2": tet32_symp2,
              "tet2": lambda: tet2_forward(n=args.adj_n, steps=args.tet2_steps),
              "adjoint": lambda: adjoint16(n=args.adj_n, nshots=args.adj_shots, steps=args.adj_steps,
                                           fd_elements=args.adj_fd, order=args.adj_order,
                                           nsnap=min(64, args.adj_steps), fd_n=args.adj_fd_n or None,
                                           tf_backward=not args.adj_no_tf)}[args.only]
        print(json.dumps(fn()))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
