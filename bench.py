#!/usr/bin/env python
"""DOF-steps/s of the scatter wave-propagation time loop on GB300.

Workload (plain method at scale): box 60 x 40 x 30 m, structured hexa8 at 0.5 m
(120 x 80 x 60 = 576,000 elements, 1,793,583 equations), two layers (top 5 m: E = 30 MPa,
nu = 0.3, rho = 1800; below: E = 150 MPa, nu = 0.25, rho = 2000), Lysmer dashpots on the
sides and base, Rayleigh 2 % at 1 and 50 Hz, moving point load 100 kN at 40 km/h along x on
the surface, dt = 5e-5 s, FP64, velocities recorded at 50 surface receivers.  One bench step
is one Newmark time step (graph launch: force, predictor, residual, device-side PCG loop,
update).  Synthetic seeded inputs; no dataset.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl gb300|reference]
    python bench.py --section batched|ragged|adjoint|csr [--dims nx,ny,nz]   # one added workload (--dims: a
                                                                             # smaller box for the batched and csr ones)

Prints one JSON line.  --impl reference times the CPU restatement of the reference path
(oracle/: numpy assembly + C Newmark/PCG loop on all host threads) on the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DOF-steps/s batched vs single-solve on GB300 at ≤1e-5 rel err; adjoint/fwd cost"
DT = 5e-5
N_T = 10001  # 10,000 steps
DIMS = (120, 80, 60, 0.5)
MATERIALS = {"lower": {"density": 2000.0, "Young": 150e6, "poisson": 0.25},
             "upper": {"density": 1800.0, "Young": 30e6, "poisson": 0.3}}
LAYERS = [(0.0, "lower"), (35.0, "upper")]
SETTINGS = {"int_order": 2, "damping": [1, 0.02, 50, 0.02], "absorbing_BC": [1, 1], "absorbing_BC_stiff": 1e3}
LOAD = {"type": "moving_at_plane", "force": [0.0, -100e3, 0.0], "speed": 40 / 3.6, "direction": [1, 0],
        "start_coord": [5.25, -15.25], "time": (N_T - 1) * DT}
N_REC = 50


def workload(dims=DIMS):
    from scatter_gb300 import meshgen
    from scatter_gb300.validator import ValidateLoad

    nx, ny, nz, h = dims
    model = meshgen.box_model(nx, ny, nz, h, layers=LAYERS, bottom="020", x_faces="200", z_faces="002")
    load = dict(LOAD)
    ValidateLoad.validate(load)
    time_grid = np.linspace(0, load["time"], int(np.ceil(load["time"] / DT) + 1))
    top_ids = model.top_nodes()
    rng = np.random.default_rng(0)
    rec_nodes = np.sort(rng.choice(top_ids, size=min(N_REC, len(top_ids)), replace=False))
    rec_eq = model.eq_nb_dof[model.node_index()[rec_nodes], 1].astype(np.int64)
    return model, load, time_grid, rec_eq


def workload_config(model, dims=DIMS):
    """The workload's description, identical in both arms' lines."""
    return {"workload": "plain Newmark FP64, box 60x40x30 m hexa8 0.5 m (120x80x60 el), 2 layers, "
                        "Lysmer sides+base, moving 100 kN at 40 km/h, dt 5e-5" if dims == DIMS
            else f"profiling case: box {dims[0]}x{dims[1]}x{dims[2]} hexa8 0.5 m, same physics",
            "n_eq": int(model.number_eq), "elements": int(len(model.elem)), "receivers": N_REC,
            "parallelism": "replicas", "l2": "inputs larger than L2 (matrices 5.1 GB), no flush"}


def force_table(model, load, time_grid):
    from scatter_gb300.force_external import Force

    F = Force()
    F.initialise_load(load, time_grid, model, None, top_surface_elements=model.get_top_surface())
    return F.table


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(name="k_spmv_pair_box120x80x60.md"):
    """dram bytes per launch of an SpMV kernel from its committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith("dram_bytes_per_launch_full_size:"):
            return float(line.split(":")[1])
    return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline_run(n, rowptr, cols, M, C, K, table, rec_eq, target_s=20.0, max_steps=None, dt=DT):
    """Oracle C Newmark/PCG on the host cores, bounded to ~target_s of work.  Returns the
    baseline record and the receiver velocities after steps 1 .. steps + 1 (from rest)."""
    from oracle import cpu

    s = cpu.NewmarkCPU.from_csr(n, rowptr, cols, M, C, K, dt)
    t0 = time.perf_counter()
    v1, _ = s.run(0, 1, table.f_ptr, table.f_eq, table.f_val, rec_eq)
    t1 = time.perf_counter() - t0
    steps = int(max(2, min(200, target_s / max(t1, 1e-6))))
    if max_steps:
        steps = min(steps, max_steps)
    t0 = time.perf_counter()
    vs, its = s.run(1, steps, table.f_ptr, table.f_eq, table.f_val, rec_eq)
    el = time.perf_counter() - t0
    rec = {"value": n * steps / el, "unit": "DOF-steps/s", "cores": cpu.threads(), "kind": "port",
           "sample": f"{steps} Newmark steps (steps 1..{steps}) of the same workload from rest, Jacobi-PCG "
                     f"per step to rtol 1e-12 started from the previous acceleration ({its / steps:.1f} "
                     f"iterations per step), {cpu.threads()} OpenMP threads, {el:.1f} s"}
    return rec, np.vstack([v1, vs])


PARITY_RTOL = 1e-8  # receiver velocities, GPU loop vs the CPU port from rest (both PCG to rtol 1e-12)


def parity_record(v_gpu, v_cpu):
    """Relative L2 of the receiver velocities over the steps both legs ran (rows = steps 1..)."""
    k = min(len(v_gpu), len(v_cpu))
    a, b = v_gpu[:k], v_cpu[:k]
    rel = float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    return {"rel_l2": rel, "steps": k, "receivers": int(a.shape[1]), "rtol": PARITY_RTOL, "ok": rel <= PARITY_RTOL,
            "against": "the CPU port (oracle C Newmark/Jacobi-PCG, FP64) on the same workload from rest"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_gb300(args):
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from scatter_gb300 import _native, replicas
    from scatter_gb300.solvers import NodeBlockNewmark
    from scatter_gb300.system_matrix import GenerateMatrix

    _native.load()
    t_setup = time.perf_counter()
    dims = tuple(int(x) for x in args.dims.split(",")) + (0.5,) if args.dims else DIMS
    model, load, time_grid, rec_eq = workload(dims)
    table = force_table(model, load, time_grid)
    t_host = time.perf_counter() - t_setup
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g = GenerateMatrix(model.number_eq, SETTINGS["int_order"])
    g.generate_stiffness_and_mass(model, MATERIALS)
    g.absorbing_boundaries(model, MATERIALS, SETTINGS["absorbing_BC"], SETTINGS["absorbing_BC_stiff"])
    g.damping_Rayleigh(SETTINGS["damping"])
    torch.cuda.synchronize()
    t_assembly = time.perf_counter() - t0
    n = model.number_eq
    K_steps, W = args.steps, args.warmup
    if W + K_steps + 1 > len(time_grid):
        raise SystemExit("steps + warmup exceed the 10,000-step load history")
    t0 = time.perf_counter()
    solver = NodeBlockNewmark(g, DT)
    torch.cuda.synchronize()
    t_solver_setup = time.perf_counter() - t0
    solver.set_force(table)
    solver.set_output(1, rec_eq, len(time_grid), what=("v",))
    solver.initial_acceleration()
    solver.run(0, W)
    rc, it_w, _ = solver.status()
    a32_w, switched_w, restarts_w, _ = solver.fp32_matrix_status()
    _, capped_w = solver.warm_start_status()
    torch.cuda.synchronize()
    replicas.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record()
        solver.run(W, W + K_steps)
        e1.record()
        torch.cuda.synchronize()
    replicas.barrier()
    ms = e0.elapsed_time(e1)
    rc, it_all, it_max = solver.status()
    if rc != 0:
        raise SystemExit(f"solver status {rc} during the timed region")
    iters = it_all - it_w
    a32_all, switched_all, restarts_all, lo_norm = solver.fp32_matrix_status()
    order_end, capped_all = solver.warm_start_status()
    a32_steps, switched, restarts = a32_all - a32_w, switched_all - switched_w, restarts_all - restarts_w
    # every rank advances its own replica: the job's rate is all ranks' DOF-steps over the
    # longest rank's time
    ms, value = replicas.job_rate(ms, n * K_steps, device="cuda")

    # dominant kernel: the PCG block SpMV in the form most timed steps ran (pair planes, or the
    # FP32 matrix alone), timed standalone on the solver's stream; both forms are reported
    ms_pair, bytes_pair = solver.time_spmv(20)
    ms_a32, bytes_a32 = solver.time_spmv(20, a32=True)
    use_a32 = 2 * a32_steps > K_steps
    ms_spmv, bytes_spmv = (ms_a32, bytes_a32) if use_a32 else (ms_pair, bytes_pair)
    peak, peak_kind = peaks()
    achieved = bytes_spmv / (ms_spmv * 1e-3) / 1e9
    traffic = profile_traffic("k_spmv_a32_box120x80x60.md" if use_a32 else "k_spmv_pair_box120x80x60.md")
    v_gpu = solver.outputs()["v"][1:W + K_steps + 1]  # receiver velocities after steps 1 .. W + K
    residual_fp64 = solver.residual_fp64()
    solver.close()

    # the same steps in IEEE FP64 throughout the PCG (what the default arithmetic saves)
    fp64 = None if args.no_e2e else ieee_fp64_run(g, table, rec_eq, W, K_steps, n, v_gpu)
    # end to end through the drop-in call: the same steps as the timed region, from a fresh
    # solver given the same warm-up
    e2e = None if args.no_e2e else e2e_run(g, table, time_grid, rec_eq, W, K_steps, n)
    if e2e is not None:
        e2e["cg_iters_per_step_device_leg"] = iters / K_steps
    # the added explicit scheme (lumped mass, one fused kernel per step) on the same model
    explicit = explicit_run(g, table, rec_eq, K_steps, W, n)
    host_csr = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        host_csr = (g.pattern.rowptr.cpu().numpy(), g.pattern.cols.cpu().numpy(),
                    *(x.cpu().numpy() for x in (g.M_d, g.C_d, g.K_d)))
    nnz = int(g.pattern.nnz)
    del g
    batched = None if args.no_batched else batched_run(min(K_steps, 2990), W)
    ragged = None if args.no_ragged else ragged_run(min(K_steps, 1990), W)
    adjoint = None if args.no_adjoint else adjoint_run()

    out = {"metric": METRIC, "value": value, "unit": "DOF-steps/s", "n_gpus": ws, "steps": K_steps, "warmup": W,
           "ms_per_step": ms / K_steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic (seeded structured mesh, moving point load)",
           "config": workload_config(model, dims),
           "solver": "Newmark beta=1/4 gamma=1/2; per step PCG (FSAI preconditioner, FP16 factor), warm start "
                     "extrapolating the accelerations, order adapted on the device, rtol 1e-12; node-block operator, "
                     "SpMV products in FP32 pairs, on the FP32 matrix (A's hi parts) in steps where the bound "
                     "on its error keeps the true residual within rtol; residual, dot products and state FP64",
           "nnz": nnz, "cg_iters_per_step": iters / K_steps, "cg_iters_max": it_max,
           "residual": "FP64 (handed over)" if residual_fp64 else "FP32 pairs on the K pair planes",
           "setup_s": {"host_mesh_and_loads": round(t_host, 2), "gpu_assembly_lysmer_rayleigh": round(t_assembly, 3),
                       "gpu_solver_setup_fsai": round(t_solver_setup, 3)},
           "fsai_fallback_rows": solver.fsai_fallback_rows,
           "fp32_matrix": {"timed_steps_started": a32_steps, "timed_steps_switched": switched,
                           "restarts": restarts, "lo_norm_bound": lo_norm},
           "ieee_fp64": fp64,
           "warm_start": {"order_at_end": order_end, "timed_steps_capped": capped_all - capped_w},
           "gpu_launches": 9 * K_steps + 5 * iters,
           "roofline": {"bound": "hbm",
                        "kernel": ("nb::k_spmv_a32 (PCG w = Ah p, the FP32 matrix, 3x3 node blocks, pair products)"
                                   if use_a32 else
                                   "nb::k_spmv_pair (PCG w = A p, 3x3 node blocks, FP32-pair products)"),
                        "achieved": achieved,
                        "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                        "traffic": traffic, "bytes_per_launch": bytes_spmv, "ms_per_launch": ms_spmv,
                        "forms": {"pair": {"ms_per_launch": ms_pair, "bytes_per_launch": bytes_pair},
                                  "a32": {"ms_per_launch": ms_a32, "bytes_per_launch": bytes_a32}}},
           "clocks": clk.summary(), "e2e": e2e, "explicit_lumped": explicit, "batched": batched,
           "ragged": ragged, "adjoint": adjoint}
    # CPU baseline (rank 0 only, N = 1): the oracle's C loop on the host cores, from rest, and
    # the GPU loop's receiver velocities over the same steps checked against it
    if rank == 0 and ws == 1 and not args.no_cpu:
        out["cpu_baseline"], v_cpu = cpu_baseline_run(n, *host_csr, table, rec_eq, target_s=args.cpu_seconds)
        out["parity"] = parity_record(v_gpu, v_cpu)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()
    if "parity" in out and not out["parity"]["ok"]:
        raise SystemExit(f"parity failed: receiver velocities differ from the CPU port by {out['parity']['rel_l2']:.3e}")


def explicit_run(g, table, rec_eq, k, w, n):
    """DOF-steps/s of the explicit lumped-mass scheme (no reference counterpart) on the model."""
    import torch

    from scatter_gb300.explicit import critical_time_step
    from scatter_gb300.solvers import NodeBlockNewmark

    dtc = critical_time_step(g)
    s = NodeBlockNewmark(g, DT, precond="jacobi")
    s.set_force(table)
    s.set_output(1, rec_eq, len(table.f_ptr) - 1, what=("v",))
    tpr = s.tune_explicit()[0]  # the step kernel's threads per row, register budget and load policy
    s.run_explicit(0, w)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    s.run_explicit(w, w + k)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ms_k = s.time_explicit(20)
    d2 = g.dim * g.dim
    sell_entries = int(s.g.adj.numel())  # stored blocks (sliced-ELL adds row padding)
    bytes_step = sell_entries * (8 * d2 + 4) + g.n_nodes * g.dim * 8 * 6
    s.close()
    return {"value": n * k / (ms / 1e3), "unit": "DOF-steps/s", "ms_per_step": ms / k, "steps": k,
            "dt": DT, "dt_critical_bound": dtc, "kernel_ms": ms_k,
            "kernel_gbs": bytes_step / (ms_k * 1e-3) / 1e9,
            "threads_per_row": tpr,
            "note": "central difference, row-sum lumped mass (no reference counterpart); u, v, K w in FP32 (hi, lo) "
                    "pairs, FP64 at the run boundary; step kernel shape tuned (threads per row, register budget, "
                    "load policy)"}


def _top_receivers(model, n, seed):
    top = model.top_nodes()
    rng = np.random.default_rng(seed)
    nodes = np.sort(rng.choice(top, size=min(n, len(top)), replace=False))
    return model.eq_nb_dof[model.node_index()[nodes], 1].astype(np.int64)


def _top_centre(model):
    top = model.top_nodes()
    X = model.nodes[model.node_index()[top], 1:]
    c = 0.5 * (X.min(axis=0) + X.max(axis=0))
    return int(top[np.argmin(((X[:, [0, 2]] - c[[0, 2]]) ** 2).sum(axis=1))])


def _events():
    import torch

    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def batched_run(k, w, R=256, dims=(80, 40, 20)):
    """Batching workload: R = 256 seeded log-normal Young's modulus realisations (mean 50 MPa,
    CoV 0.25, Gaussian covariance, correlation lengths 5 / 1 / 5 m in x / y (vertical) / z),
    nu = 0.3, rho = 1900, box 40 x 20 x 10 m hexa8 at 0.5 m (80 x 40 x 20 elements), Lysmer
    sides and base, Ricker 20 Hz at the top centre; all realisations advanced by one kernel
    per step, against the plain FP64 explicit GPU path run once for one realisation."""
    import torch

    from scatter_gb300 import device as dv
    from scatter_gb300 import meshgen
    from scatter_gb300.batched import BatchedExplicit
    from scatter_gb300.force_external import ricker_table
    from scatter_gb300.random_fields import element_centroids, lognormal_fields
    from scatter_gb300.solvers import NodeBlockNewmark
    from scatter_gb300.system_matrix import GenerateMatrix

    m = meshgen.box_model(*dims, 0.5, bottom="020", x_faces="200", z_faces="002")
    n_t = 3001
    if w + k + 1 > n_t:
        raise SystemExit("batched steps + warmup exceed the 3000-step history")
    tg = np.arange(n_t) * DT
    table = ricker_table(m, _top_centre(m), -10e3, 20.0, 0.05, tg)
    rec_eq = _top_receivers(m, N_REC, 1)
    nu, rho = 0.3, 1900.0
    young = lognormal_fields(element_centroids(m), seed=2024, R=R, lengths=(5.0, 1.0, 5.0), mean=50e6, sd=12.5e6)
    n = int(m.number_eq)
    b = BatchedExplicit(m, young, nu, rho, SETTINGS["damping"], SETTINGS["absorbing_BC"],
                        SETTINGS["absorbing_BC_stiff"], DT)
    b.set_force(table)
    b.set_output(1, rec_eq, n_t)
    rpt, tpb, tuned_ms, grid_kernel = b.config()
    b.run(0, w)
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    b.run(w, w + k)
    e1.record()
    torch.cuda.synchronize()
    ms_b = e0.elapsed_time(e1)
    vb_all = b.velocities()[: w + k + 1]  # [step, receiver, realisation]
    # the tensor-core kernel (a tuner candidate) timed on its own at its best column segment
    tc_ms = None
    if b.column_tables is not None:
        nzp = b.column_tables[2]
        tc_ms = {}
        for seg in sorted({nzp, -(-nzp // 2), -(-nzp // 3)}):
            b.set_tensor_core_shape(seg)
            b.run(0, 3)
            e0, e1 = _events()
            e0.record()
            b.run(3, 13)
            e1.record()
            torch.cuda.synchronize()
            b.status()
            tc_ms[seg] = e0.elapsed_time(e1) / 10
    young_h = dv.host(young).astype(float)
    b.close()
    del b
    n_el = len(m.elem)

    def single_run(r, timed):
        """Realisation r through the plain FP64-class explicit GPU path (its own assembly)."""
        g = GenerateMatrix(n, SETTINGS["int_order"])
        g.generate_stiffness_and_mass(m, None, element_props=(young_h[:, r], np.full(n_el, nu), np.full(n_el, rho)))
        g.absorbing_boundaries(m, None, SETTINGS["absorbing_BC"], SETTINGS["absorbing_BC_stiff"])
        g.damping_Rayleigh(SETTINGS["damping"])
        s = NodeBlockNewmark(g, DT, precond="jacobi")
        s.set_force(table)
        s.set_output(1, rec_eq, n_t, what=("v",))
        tpr = s.tune_explicit()[0] if timed else None  # the single solve at its own best shape
        s.run_explicit(0, w)
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record()
        s.run_explicit(w, w + k)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        vs = dv.host(s.out["v"]).reshape(n_t, len(rec_eq))[: w + k + 1]
        s.close()
        return vs, ms, tpr

    # the checked realisations: eight spread over the batch, the first one timed
    picks = np.unique(np.linspace(0, R - 1, min(8, R)).round().astype(int))
    rels = {}
    for r in picks:
        vs, ms, tpr = single_run(int(r), r == picks[0])
        if r == picks[0]:
            ms_s, single_tpr = ms, tpr
        vb = vb_all[:, :, r]
        rels[int(r)] = float(np.linalg.norm(vb - vs) / max(np.linalg.norm(vs), 1e-300))
    vb_rate = n * R * k / (ms_b / 1e3)
    single = n * k / (ms_s / 1e3)
    return {"value": vb_rate, "unit": "DOF-steps/s", "single_solve": single, "speedup_vs_single": vb_rate / single,
            "realisations": R, "n_eq": n, "elements": n_el, "steps": k, "warmup": w, "ms_per_step": ms_b / k,
            "single_ms_per_step": ms_s / k, "rel_l2_vs_fp64_max": max(rels.values()),
            "rel_l2_vs_fp64": rels, "rel_l2_rtol": 1e-5,
            "tuned_shape": {"kernel": BatchedExplicit.KERNELS[grid_kernel],
                            ("column_segment_points" if grid_kernel == 2 else "realisations_per_thread"): rpt,
                            "threads_per_block": tpb, "tuned_ms": tuned_ms},
            "tensor_core_kernel_ms_per_step": tc_ms,
            "workload": "256 log-normal E realisations, box 40x20x10 m hexa8 0.5 m, Lysmer, Ricker 20 Hz, dt 5e-5",
            "single": "plain FP64-class explicit GPU path (node-block graph, threads per row tuned: "
                      f"{single_tpr}), realisation 0 timed, same steps; receiver velocities of realisations "
                      f"{[int(r) for r in picks]} checked against their own single solves"}


def ragged_run(k, w, n_meshes=64, seed=4, hexa_edges=(10, 80), tetra_edges=(5, 40)):
    """Ragged batching: 64 seeded meshes of uneven size -- hexa8 boxes with 10-80 elements per
    axis and tetra10 boxes (5-40 hexes per axis, each split into 6 quadratic tets) at 0.5 m,
    homogeneous E in [20, 200] MPa, nu in [0.2, 0.35], rho in [1700, 2100] per mesh, base fixed
    and lateral rollers, Ricker 20 Hz at each top centre, dt 5e-5 -- advanced together by one
    matrix-free kernel per step (FP32 products, pair accumulators; threads per block
    autotuned), against every mesh advanced alone through the same path."""
    import torch

    from scatter_gb300.ragged import RaggedBatch, mesh_specs

    specs = mesh_specs(n_meshes, seed, hexa_edges=hexa_edges, tetra_edges=tetra_edges)
    n_t = 2001
    tg = np.arange(n_t) * DT
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    t0 = time.perf_counter()
    r = RaggedBatch(specs, SETTINGS["damping"], DT, tg)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    used_gb = (free0 - torch.cuda.mem_get_info()[0]) / 1e9
    r.set_output(1, n_t)
    r.run(0, w)
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    r.run(w, w + k)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    n_eq, n_dof_slots, tuned = r.n_eq, 3 * r.n_nodes, r.tuned
    r.close()
    del r
    # every mesh alone, the same path and steps
    seq_ms = 0.0
    k_alone = min(k, 40)
    for sp in specs:
        a = RaggedBatch([sp], SETTINGS["damping"], DT, tg)
        a.set_output(1, n_t)
        a.run(0, w)
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record()
        a.run(w, w + k_alone)
        e1.record()
        torch.cuda.synchronize()
        seq_ms += e0.elapsed_time(e1) / k_alone
        a.close()
    value = n_eq * k / (ms / 1e3)
    seq = n_eq / (seq_ms / 1e3)
    return {"value": value, "unit": "DOF-steps/s", "meshes": n_meshes, "n_eq": n_eq, "slots": n_dof_slots,
            "hexa8": sum(s["element"] == "hexa8" for s in specs), "tetra10": sum(s["element"] == "tetra10" for s in specs),
            "steps": k, "ms_per_step": ms / k, "sequential_ms_per_step": seq_ms, "sequential": seq,
            "speedup_vs_sequential": value / seq, "threads_per_block": tuned[0], "setup_s": round(setup_s, 1),
            "device_memory_gb": round(used_gb, 1),
            "workload": f"64 seeded meshes: hexa8 edges {hexa_edges[0]}-{hexa_edges[1]}, tetra10 (6 tets per hex) "
                        f"{tetra_edges[0]}-{tetra_edges[1]} hexes per axis, 0.5 m, Ricker 20 Hz, dt 5e-5",
            "arithmetic": "matrix-free: FP32 element products, u and v in FP32 (hi, lo) pairs"}


def csr_run(k, w, dims=(60, 30, 40, 0.5)):
    """The Newmark loop on scipy matrices (the CSR layout, Jacobi-PCG with the adaptive warm
    start): a box of the benchmark's physics (default 30 x 15 x 20 m, hexa8 at 0.5 m).  The
    standalone SpMV timing runs first, before any graph launch, so a profiler can capture it."""
    import ctypes

    import torch

    from scatter_gb300 import _native as nat
    from scatter_gb300.solvers import NewmarkGPU, _device_matrices
    from scatter_gb300.system_matrix import GenerateMatrix

    model, load, tg, rec_eq = workload(dims)
    table = force_table(model, load, tg)
    g = GenerateMatrix(model.number_eq, 2)
    g.generate_stiffness_and_mass(model, MATERIALS)
    g.absorbing_boundaries(model, MATERIALS, SETTINGS["absorbing_BC"], SETTINGS["absorbing_BC_stiff"])
    g.damping_Rayleigh(SETTINGS["damping"])
    pat, Md, Cd, Kd = _device_matrices(g.M, g.C, g.K)
    s = NewmarkGPU(pat, Md, Cd, Kd, DT)
    ms, nb = ctypes.c_float(), ctypes.c_int64()
    nat.call("sc_newmark_time_spmv", s.h, 20, ctypes.byref(ms), ctypes.byref(nb))
    k = max(1, min(k, len(tg) - 1 - w))
    s.set_force(table)
    s.set_output(1, rec_eq, len(tg), what=("v",))
    s.initial_acceleration()
    s.run(0, w)
    _, it0, _ = s.status()
    e0, e1 = _events()
    e0.record()
    s.run(w, w + k)
    e1.record()
    torch.cuda.synchronize()
    rc, it1, it_max = s.status()
    step_ms = e0.elapsed_time(e1) / k
    s.close()
    n = model.number_eq
    return {"value": n / (step_ms / 1e3), "unit": "DOF-steps/s", "n_eq": n, "nnz": int(pat.nnz), "steps": k,
            "ms_per_step": step_ms, "pcg_iterations_per_step": (it1 - it0) / k, "max_iterations": it_max,
            "status": rc, "spmv_us": ms.value * 1e3, "spmv_bytes": nb.value,
            "spmv_gbs": nb.value / ms.value / 1e6,
            "workload": f"box {dims[0]}x{dims[1]}x{dims[2]} hexa8 {dims[3]} m, benchmark physics, scipy CSR "
                        "matrices, Jacobi-PCG"}


def adjoint_run(n_steps=4000, checkpoint=200, n_fd=20):
    """Differentiation workload: misfit of vertical surface velocities at 25 receivers w.r.t.
    per-element E and rho, box 20 x 10 x 20 m (x / y vertical / z) hexa8 at 0.5 m (32,000
    elements), target from a seeded log-normal E field (CoV 0.3, correlation 3 m), evaluated
    at a homogeneous 60 MPa guess; 4000 steps, checkpoint every 200.  Reports the cost of one
    gradient against one forward solve, and central differences (h = 1e-6 relative) on
    n_fd elements (half E, half rho) drawn from those with the largest gradients."""
    import torch

    from scatter_gb300 import meshgen
    from scatter_gb300.adjoint import ExplicitAdjoint
    from scatter_gb300.force_external import ricker_table
    from scatter_gb300.random_fields import element_centroids, lognormal_fields

    m = meshgen.box_model(40, 20, 40, 0.5, bottom="020", x_faces="200", z_faces="002")
    tg = np.arange(n_steps + 1) * DT
    table = ricker_table(m, _top_centre(m), -10e3, 20.0, 0.05, tg)
    rec_eq = _top_receivers(m, 25, 5)
    n_el = len(m.elem)
    nu, rho = np.full(n_el, 0.3), np.full(n_el, 1900.0)
    from scatter_gb300 import device as dv

    E_true = dv.host(lognormal_fields(element_centroids(m), seed=77, R=1, lengths=(3.0, 3.0, 3.0), mean=60e6,
                                      sd=18e6))[:, 0].astype(float)
    E0 = np.full(n_el, 60e6)
    A = ExplicitAdjoint(m, nu, SETTINGS["damping"], SETTINGS["absorbing_BC"], SETTINGS["absorbing_BC_stiff"], DT,
                        n_steps, rec_eq, table, checkpoint=checkpoint)
    p = A.prepare(E_true, rho)
    target = p.forward()
    p.close()
    p = A.prepare(E0, rho)
    p.forward()  # builds the explicit graphs
    s = p.solver
    s.u.zero_()
    s.v.zero_()
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    s.run_explicit(0, n_steps)
    e1.record()
    torch.cuda.synchronize()
    ms_f = e0.elapsed_time(e1)
    kernel_ms = s.time_explicit(20)  # the step kernel alone, back-to-back launches
    p.gradient(target)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J, gE, gR = p.gradient(target)
    ms_a = (time.perf_counter() - t0) * 1e3
    phases = p.timings()
    v0 = p.forward()
    p.close()

    def misfit(E, r):
        q = A.prepare(E, r)
        v = q.forward()
        q.close()
        return 0.5 * float(((v[1:] - target[1:]) ** 2).sum())

    rng = np.random.default_rng(11)
    worst = 0.0
    checks = []
    for kind, grad in (("E", gE), ("rho", gR)):
        top = np.argsort(-np.abs(grad))[: max(n_el // 20, n_fd)]
        for e in rng.choice(top, size=n_fd // 2, replace=False):
            base = E0 if kind == "E" else rho
            h = 1e-6 * base[e]
            up, dn = base.copy(), base.copy()
            up[e] += h
            dn[e] -= h
            fd = ((misfit(up, rho) - misfit(dn, rho)) if kind == "E" else (misfit(E0, up) - misfit(E0, dn))) / (2 * h)
            err = abs(fd - grad[e]) / abs(grad[e])
            worst = max(worst, err)
            checks.append([kind, int(e), float(grad[e]), float(fd)])
    return {"adjoint_over_forward": ms_a / ms_f, "forward_ms": ms_f, "gradient_ms": ms_a,
            "gradient_phases_ms": {"forward_with_checkpoints": phases[0], "recompute_last_segment": phases[1],
                                   "backward_with_recompute": phases[2], "reverse_sweep": phases[3]},
            "reverse_sweep": "each backward step fused with a recompute step of the previous segment (one kernel "
                             "per pair of steps); element gradients once per segment", "explicit_kernel_ms": kernel_ms, "misfit": J,
            "misfit_check": 0.5 * float(((v0[1:] - target[1:]) ** 2).sum()), "n_eq": int(m.number_eq),
            "elements": n_el, "steps": n_steps, "checkpoint": checkpoint, "fd_max_rel_err": worst, "fd_checks": len(checks),
            "timing": "forward: CUDA events around the explicit run; gradient: host wall clock around the whole "
                      "sc_nb_adjoint call (forward with checkpoints, recompute, backward, graph set-up, copies)"}


def ieee_fp64_run(g, table, rec_eq, w, k, n, v_ref):
    """The same steps with IEEE FP64 throughout the PCG (FP64 SpMV and FP64 residual, no FP32
    matrix): what the default arithmetic saves, and how far its receiver velocities are from
    the all-FP64 ones."""
    import torch

    from scatter_gb300.solvers import NodeBlockNewmark

    s = NodeBlockNewmark(g, DT, spmv="fp64", residual="fp64")
    s.set_force(table)
    s.set_output(1, rec_eq, len(table.f_ptr) - 1, what=("v",))
    s.initial_acceleration()
    s.run(0, w)
    rc, it_w, _ = s.status()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    s.run(w, w + k)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    rc, it_all, _ = s.status()
    v = s.outputs()["v"][1:w + k + 1]
    s.close()
    if rc != 0:
        raise SystemExit(f"FP64 solver status {rc}")
    rel = float(np.linalg.norm(v - v_ref) / max(np.linalg.norm(v), 1e-300))
    return {"value": n * k / (ms / 1e3), "unit": "DOF-steps/s", "ms_per_step": ms / k, "steps": k,
            "cg_iters_per_step": (it_all - it_w) / k,
            "rel_l2_default_vs_fp64": rel,
            "note": "PCG SpMV (A as FP64) and step residual in IEEE FP64, same warm start, preconditioner and "
                    "tolerance; receiver velocities of the default arithmetic compared with these"}


def e2e_run(g, table, time_grid, rec_eq, w, k, n):
    """The metric end to end through the drop-in call, over the same steps as the timed region.

    A fresh solver is driven as the reference drives PuggleSolvers' NewmarkExplicit
    (scatter/scatter.py:121-159): ``calculate(M, C, K, F, t0, t1)``, with the GenerateMatrix
    passed for M, C and K (the form this package's scatter() uses; the scipy matrices it
    hands out reach the same solver, but downloading three 141.7 M-entry matrices to the host
    is set-up cost outside this metric).  The untimed first call (steps 0 .. w)
    builds the solver and runs the same warm-up as the device-timed leg; the timed region is
    then k calls of one step each, w .. w + k, each copying that step's force values host ->
    device from pinned memory and queueing the device -> host copies of its receiver outputs
    (u, v, a) and of the run's status into pinned buffers; a call's outputs reach the solver's
    host arrays at the next call (the last one's when the timed region ends)."""
    import torch

    from scatter_gb300.solvers import NewmarkExplicit

    if k <= 0:
        return None
    M = C = K = g
    s = NewmarkExplicit()
    s.output_interval = 1
    s.initialise(n, time_grid)
    s.force_table = table
    s.receivers = rec_eq
    s.stream_force = True
    s.update(0)
    s.calculate(M, C, K, None, 0, w)
    dev = s.device_solver
    rc, it_w, _ = dev.status()
    h2d0 = dev.force.h2d_bytes
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    wall0 = time.perf_counter()
    ev0.record()
    for t in range(w, w + k):
        s.calculate(M, C, K, None, t, t + 1)
    ev1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    ms = ev0.elapsed_time(ev1)
    rc, it_all, _ = dev.status()
    h2d = dev.force.h2d_bytes - h2d0
    s.close()
    return {"value": n * k / (ms / 1e3), "unit": "DOF-steps/s", "h2d_bytes_per_step": h2d / k,
            "d2h_bytes_per_step": 3 * len(rec_eq) * 8, "steps": k, "first_step": w, "ms_per_step": ms / k,
            "host_wall_s": wall, "cg_iters_per_step": (it_all - it_w) / k, "preconditioner": s.preconditioner,
            "api": "NewmarkExplicit.calculate(matrix, matrix, matrix, F, t, t + 1) once per step (GenerateMatrix "
                   "for M, C, K; force values streamed from pinned host memory; each call queues the copies of its "
                   "receiver u, v, a and of the run's status to pinned host buffers, delivered at the next call)"}


def run_reference(args):
    """CPU restatement of the reference path on the host cores (oracle: numpy element
    integration + element-order assembly + Lysmer + Rayleigh, C Newmark/PCG loop)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import scipy.sparse as sp

    from oracle import assembly as asm
    from oracle import elements as el
    from oracle import lysmer

    t0 = time.perf_counter()
    model, load, time_grid, rec_eq = workload()
    table = force_table(model, load, time_grid)
    n = model.number_eq
    idx = model.node_index()[model.elem]
    X = model.nodes[:, 1:][idx]
    names = {int(r[1]): r[2] for r in model.materials}
    mi = model.materials_index
    E = np.array([MATERIALS[names[int(i)]]["Young"] for i in mi])
    nu = np.array([MATERIALS[names[int(i)]]["poisson"] for i in mi])
    rho = np.array([MATERIALS[names[int(i)]]["density"] for i in mi])
    rows, cols, kv, mv = [], [], [], []
    eq = model.eq_nb_elem
    # the oracle integrates each distinct element (node offsets and material) once; every
    # element of the structured mesh is one of them, so its matrices are exactly those
    off = np.round((X - X[:, :1, :]).reshape(len(X), -1) * 1e9).astype(np.int64)
    sig = np.c_[off, np.asarray(mi, dtype=np.int64)]
    _, first, inv = np.unique(sig, axis=0, return_index=True, return_inverse=True)
    inv = inv.ravel()
    Ke_u, Me_u = el.element_matrices("hexa8", X[first], E[first], nu[first], rho[first])
    for s in range(0, len(X), 20000):
        Ke, Me = Ke_u[inv[s:s + 20000]], Me_u[inv[s:s + 20000]]
        e = eq[s:s + 20000]
        ok = ~np.isnan(e)
        ei = np.where(ok, e, -1).astype(np.int64)
        R = np.broadcast_to(ei[:, :, None], Ke.shape)
        Cc = np.broadcast_to(ei[:, None, :], Ke.shape)
        m = (R >= 0) & (Cc >= 0)
        rows.append(R[m])
        cols.append(Cc[m])
        kv.append(Ke[m])
        mv.append(Me[m])
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    K0 = sp.coo_matrix((np.concatenate(kv), (rows, cols)), shape=(n, n)).tocsr()
    M = sp.coo_matrix((np.concatenate(mv), (rows, cols)), shape=(n, n)).tocsr()
    mdl = {"nodes": model.nodes, "elem": model.elem, "BC": model.BC, "BC_dir": model.BC_dir,
           "eq_nb_dof": model.eq_nb_dof, "element_type": "hexa8", "number_eq": n}
    Ca, Ka = lysmer.absorbing(mdl, (E, nu, rho), SETTINGS["absorbing_BC"], SETTINGS["absorbing_BC_stiff"])
    K = asm.drop_zeros(K0 + Ka)
    C = asm.rayleigh(M, K, Ca, SETTINGS["damping"])
    setup = time.perf_counter() - t0
    from oracle import cpu

    s = cpu.NewmarkCPU(M, C, K, DT)
    budget = args.cpu_seconds
    # untimed warm-up: the requested W steps, within half the time budget (at least one)
    t1 = time.perf_counter()
    s.run(0, 1, table.f_ptr, table.f_eq, table.f_val, rec_eq)
    one = time.perf_counter() - t1
    w_steps = int(max(1, min(args.warmup, budget / 2 / max(one, 1e-6))))
    if w_steps > 1:
        s.run(1, w_steps - 1, table.f_ptr, table.f_eq, table.f_val, rec_eq)  # (first step, step count)
    steps = int(max(2, min(args.steps, budget / max(one, 1e-6))))
    t1 = time.perf_counter()
    _, its = s.run(w_steps, steps, table.f_ptr, table.f_eq, table.f_val, rec_eq)
    el_s = time.perf_counter() - t1
    value = n * steps / el_s
    cb = {"value": value, "unit": "DOF-steps/s", "cores": cpu.threads(), "kind": "port",
          "sample": f"{steps} Newmark steps ({w_steps}..{w_steps + steps - 1}) of the same workload after {w_steps} "
                    f"untimed steps from rest; oracle numpy assembly "
                    f"({setup:.0f} s, untimed) + C Jacobi-PCG loop started from the previous acceleration "
                    f"({its / steps:.1f} iterations per step) on {cpu.threads()} threads, {el_s:.1f} s"}
    print(json.dumps({"metric": METRIC, "value": value, "unit": "DOF-steps/s", "n_gpus": ws, "steps": steps,
                      "warmup": w_steps, "ms_per_step": el_s / steps * 1e3, "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded structured mesh)",
                      "config": workload_config(model), "impl": "reference", "cpu_baseline": cb,
                      "e2e": {"value": value, "unit": "DOF-steps/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--dims", default="", help="nx,ny,nz of a smaller box (profiling cases)")
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-realisation batched measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint cost and FD measurement")
    ap.add_argument("--no-ragged", action="store_true", help="skip the 64-mesh ragged batching measurement")
    ap.add_argument("--section", default="all", choices=["all", "batched", "adjoint", "ragged", "csr"],
                    help="run one added workload alone and print its JSON (profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.section != "all":
        import torch

        torch.cuda.set_device(0)
        from scatter_gb300 import _native

        _native.load()
        if args.section == "batched":
            dims = tuple(int(x) for x in args.dims.split(",")) if args.dims else (80, 40, 20)
            out = batched_run(min(args.steps, 2990), args.warmup, dims=dims)
        elif args.section == "ragged":
            out = ragged_run(min(args.steps, 1990), args.warmup)
        elif args.section == "csr":
            dims = tuple(int(x) for x in args.dims.split(",")) + (0.5,) if args.dims else (60, 30, 40, 0.5)
            out = csr_run(args.steps, args.warmup, dims)
        else:
            out = adjoint_run(n_steps=args.steps, checkpoint=min(200, args.steps), n_fd=0 if args.no_cpu else 20)
        print(json.dumps({"section": args.section, **out}))
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
