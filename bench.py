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
        "cpu_baseline": {"value": value, "unit": "DOF-updates/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "DOF-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def fdtd_512(steps=60, n=512):
    """n^3 (512^3 by default) FP32 Yee step with a 10-cell CPML: device rate
    and roofline of the E kernel."""
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
    s = ems.FdtdSimulation((n, n, n), h, dt, eps0, mu0, 1, precision=ems.FP32, pml_cells=10, pml_order=3.0,
                           pml_kappa_max=1.0, pml_alpha_max=0.0, pml_reflection=1e-6)
    s.set_material(blk_eps[cell_blk], blk_sig[cell_blk])
    del cell_blk
    for q in range(4):
        c = rng.integers(20, n - 20, 3)
        s.setSource_z(tuple(int(v) for v in c), waveform=ems.WAVE_RICKER, f0=float(rng.uniform(5e9, 15e9)))
    s.run(24)          # warm-up; the handle's first run of >= 24 steps picks the launch shape
    s.run(steps)
    ms, launches = s.run_stats()
    kms, kbytes, kname = s.time_dominant_kernel(10)
    shape = s.launch_shape()
    cells = n ** 3
    s.close()
    return {"workload": f"fdtd{n}_fp32_cpml10", "steps": steps, "ms_per_step": ms / steps,
            "launch_shape": list(shape[:2]),
            "cell_updates_per_s": cells * steps / (ms * 1e-3),
            "dof_updates_per_s": 6 * cells * steps / (ms * 1e-3),
            "kernel": kname, "kernel_ms": kms, "kernel_bytes": kbytes, "kernel_gbs": kbytes / (kms * 1e-3) / 1e9}


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


def batch64(nshots=64, steps=3000, sample=8, sample_steps=300):
    """Batched forward shots: nshots cubes of side n ~ U[12,40] (6 n^3
    tetrahedra each), eps_r ~ U[1,6] per tet, one Ricker dipole each, 4th-order
    symplectic, `steps` steps, FP32, all shots advanced by the same kernels.
    Compared with the plain per-shot FP64 GPU path on `sample` of the shots
    (same time step, `sample_steps` steps, scaled to `steps`)."""
    import emsolvers_gb300 as ems
    rng = np.random.default_rng(SEED + 4)
    sides = rng.integers(12, 41, nshots)
    cells = [(int(n), int(n), int(n)) for n in sides]
    eps = [rng.uniform(1.0, 6.0, 6 * n ** 3) for n in sides]
    pos = [np.array([n, n, n]) * rng.uniform(0.3, 0.7, 3) * H for n in sides]
    rec = [np.array([n, n, n]) * rng.uniform(0.2, 0.8, 3) * H for n in sides]
    f0 = C0 / (10 * H * np.sqrt(3.5))
    b = ems.TetFemBatch(cells, H, integrator=ems.SYMP4, precision=ems.FP32, dt=0.0, cfl_fraction=0.9)
    b.set_material(np.concatenate(eps))
    for s in range(nshots):
        b.add_dipole(s, pos[s], (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0)
        b.add_receiver(s, rec[s])
    dt, _ = b.time_step()
    b.run(20)
    b.reset()
    b.run(steps)
    ms_batch, launches = b.run_stats()
    kms, kbytes, kname = b.time_dominant_kernel(20)
    block = b.launch_shape()[0]
    edges = sum(n_edges(int(n)) for n in sides)
    b.close()
    per = {ems.FP64: [], ems.FP32: []}
    pick = rng.choice(nshots, size=min(sample, nshots), replace=False)
    for prec in (ems.FP64, ems.FP32):
        for s in pick:
            one = ems.TetFemSimulation(cells[s], H, 1, ems.SYMP4, prec, dt=dt)
            one.set_material(eps[s])
            one.add_dipole(pos[s], (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0)
            one.add_receiver(rec[s])
            one.run(5)
            one.reset()
            one.run(sample_steps)
            per[prec].append(one.run_stats()[0] * steps / sample_steps)
            one.close()
    shots_batch = nshots / (ms_batch * 1e-3)
    shots_fp64 = 1.0 / (np.mean(per[ems.FP64]) * 1e-3)
    shots_fp32 = 1.0 / (np.mean(per[ems.FP32]) * 1e-3)
    return {"workload": "tet_batch64_symp4_3000", "shots": nshots, "steps": steps, "tets": int(sum(6 * sides ** 3)),
            "edges": int(edges), "order": 1, "dt_s": dt, "batch_ms": ms_batch, "launches": int(launches),
            "shots_per_s_fp32_batched": shots_batch, "shots_per_s_fp64_per_shot": shots_fp64,
            "shots_per_s_fp32_per_shot": shots_fp32, "speedup_vs_fp64_per_shot": shots_batch / shots_fp64,
            "dof_updates_per_s": edges * steps / (ms_batch * 1e-3),
            "per_shot_sample": f"{len(pick)} shots x {sample_steps} steps, scaled to {steps}",
            "kernel": kname, "kernel_us": kms * 1e3, "kernel_gbs": kbytes / (kms * 1e-3) / 1e9, "threads_per_block": block}


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


def adjoint16(n=48, nshots=16, nrec=32, steps=4000, nsnap=64, sample_steps=400):
    """Forward + adjoint misfit gradient: nshots Ricker dipole shots on an
    n^3 x 6 tet cube (true eps_r = 2 + 3 Gaussian blobs, start model 2), nrec
    receivers per shot, symp4, `steps` steps, L2 trace misfit, nsnap
    snapshots.  FP32 batched (all shots in one handle) against the plain
    per-shot FP64 GPU path, the latter timed on one shot over
    `sample_steps` steps (same segment length) and scaled to `steps`."""
    import emsolvers_gb300 as ems
    rng = np.random.default_rng(SEED + 5)
    true = blob_model(n, rng)
    start = np.full(true.size, 2.0)
    f0 = C0 / (10 * H * np.sqrt(2.0))
    src = [rng.uniform(0.2, 0.8, 3) * n * H for _ in range(nshots)]
    rec = [rng.uniform(0.1, 0.9, 3) * n * H for _ in range(nrec)]
    probe = ems.TetFemSimulation((n, n, n), H, 1, ems.SYMP4, ems.FP32, dt=0.0, cfl_fraction=0.9)
    probe.set_material(start)
    dt, _ = probe.time_step()
    probe.close()

    def handle(precision, shots, model):
        b = ems.TetFemBatch([(n, n, n)] * len(shots), H, integrator=ems.SYMP4, precision=precision, dt=dt)
        b.set_material(np.tile(model, len(shots)))
        for k, s in enumerate(shots):
            b.add_dipole(k, src[s], (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0)
            for r in rec:
                b.add_receiver(k, r)
        return b

    shots = list(range(nshots))
    b = handle(ems.FP32, shots, true)
    b.run(steps)
    obs = b.traces()
    import torch
    torch.cuda.synchronize()
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
    g32 = b.backward(tg).reshape(nshots, -1).sum(0)
    ts.append(time.perf_counter())
    wall32 = ts[-1] - t0
    stages = {"setup_s": ts[0] - t0, "forward_s": ts[1] - ts[0], "misfit_s": ts[2] - ts[1], "backward_s": ts[3] - ts[2]}
    b.close()
    # per-shot FP64 sample with the same segment length
    seg = -(-steps // nsnap)
    one = handle(ems.FP64, [0], start)
    one.set_checkpoints(-(-sample_steps // seg))
    obs0 = obs[:nrec, :sample_steps]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    one.set_material(start)
    one.time_step()                    # FP64 mass setup and stability limit, once per gradient
    t1 = time.perf_counter()
    one.reset()
    one.run(sample_steps)
    _, tg0 = ems.trace_misfit(one.traces(), obs0, ems.MISFIT_L2)
    g64_0 = one.backward(tg0)
    t2 = time.perf_counter()
    wall64 = (t1 - t0) + (t2 - t1) * steps / sample_steps
    tr64 = one.traces()
    one.close()
    # FP32 against FP64 on the same sampled shot
    one32 = handle(ems.FP32, [0], start)
    one32.set_checkpoints(-(-sample_steps // seg))
    one32.reset()
    one32.run(sample_steps)
    g32_0 = one32.backward(tg0)
    tr_err = float(np.linalg.norm(one32.traces()[..., 1:] - tr64[..., 1:]) / np.linalg.norm(tr64[..., 1:]))
    one32.close()
    g_err = float(np.linalg.norm(g32_0 - g64_0) / np.linalg.norm(g64_0))
    return {"workload": f"tet{n}_adjoint_{nshots}shots_symp4_{steps}", "tets_per_shot": int(true.size),
            "shots": nshots, "receivers_per_shot": nrec, "steps": steps, "snapshots": nsnap, "misfit": "L2",
            "order": 1, "dt_s": dt, "misfit_value": J, "grad_norm": float(np.linalg.norm(g32)),
            "fp32_batched_s": wall32, "fp32_forward_ms": fwd_ms, "fp32_stages": stages,
            "shots_per_s_fp32_batched": nshots / wall32, "shots_per_s_fp64_per_shot": 1.0 / wall64,
            "speedup_vs_fp64_per_shot": (nshots / wall32) * wall64,
            "fp64_sample": f"1 shot x {sample_steps} steps (time loop scaled to {steps}, setup once)",
            "fp64_setup_s": t1 - t0,
            "fp32_vs_fp64_trace_rel_l2": tr_err, "fp32_vs_fp64_grad_rel_l2": g_err,
            "fp32_vs_fp64_over": f"shot 0, its first {sample_steps} of {steps} steps (forward and gradient)",
            "timing": "wall clock: material upload + FP64 mass setup + recorded forward + misfit + backward"}


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
    # ---- dominant kernel roofline
    kms, kbytes, kname = sim.time_dominant_kernel(200)
    block = sim.launch_shape()[0]
    peak, peak_kind = peaks()
    achieved = kbytes / (kms * 1e-3) / 1e9
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
                     # profiles/tet_step_tet32_symp4.md (cold fill: the 8.6 MB
                     # working set is L2-resident in the timed loop)
                     "traffic": 6598656, "kernel": kname, "kernel_us": kms * 1e3, "bytes_per_launch": kbytes,
                     "threads_per_block": block, "peak_source": peak_kind},
        "clocks": clk,
        "wall_s": wall,
    }
    if rank == 0:
        if not args.no_cpu:
            secs = [cpu_oracle_rate(STEPS_PER_SOLVE, os.cpu_count() or 1)[1] for _ in range(3)]
            r = n_edges(N) * 3 * STEPS_PER_SOLVE / sum(secs)
            out["cpu_baseline"] = {"value": r, "unit": "DOF-updates/s", "cores": os.cpu_count() or 1, "kind": "port",
                                   "sample": f"three full solves ({STEPS_PER_SOLVE} time steps each), FP64 oracle, "
                                             f"{sum(secs):.1f} s"}
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
                out["adjoint16"] = adjoint16()
            except Exception as e:  # secondary measurement only
                out["adjoint16"] = {"error": str(e)}
        if not args.no_fdtd:
            try:
                out["fdtd_512"] = fdtd_512()
                out["fdtd_512"]["hbm_frac"] = out["fdtd_512"]["kernel_gbs"] / peak
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
    ap.add_argument("--only", choices=["head", "batch", "fdtd", "adjoint", "hex"],
                    help="run one secondary workload alone and print its JSON (for profiling)")
    ap.add_argument("--fdtd-n", type=int, default=512, help="FDTD cube side for --only fdtd")
    ap.add_argument("--head-steps", type=int, default=STEPS_PER_SOLVE, help="time steps for --only head")
    ap.add_argument("--batch-steps", type=int, default=3000, help="time steps for --only batch")
    ap.add_argument("--batch-sample", type=int, default=8, help="per-shot FP64 sample size for --only batch")
    ap.add_argument("--adj-n", type=int, default=48, help="cube side for --only adjoint")
    ap.add_argument("--adj-steps", type=int, default=4000, help="time steps for --only adjoint")
    ap.add_argument("--adj-shots", type=int, default=16, help="shots for --only adjoint")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        fn = {"head": lambda: head_solve(args.head_steps),
              "batch": lambda: batch64(steps=args.batch_steps, sample=args.batch_sample,
                                       sample_steps=min(300, args.batch_steps)),
              "fdtd": lambda: fdtd_512(n=args.fdtd_n), "hex": hex72,
              "adjoint": lambda: adjoint16(n=args.adj_n, nshots=args.adj_shots, steps=args.adj_steps,
                                           sample_steps=min(400, args.adj_steps))}[args.only]
        print(json.dumps(fn()))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
