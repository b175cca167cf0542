"""The CPU baseline of bench.py (the oracle's C Newmark/PCG loop on the host cores): its
record on a small golden system, and the same loop's history against the oracle's direct
solve."""
import numpy as np

from helpers import oracle_system, rel_l2


def _system():
    from oracle import cpu, loads
    from scatter_gb300.solvers import ForceTable

    model, spec, M, C, K, _, _ = oracle_system("column_hexa8_abs")
    load = dict(spec["load"])
    time = loads.time_grid(load["time"], spec["dt"])
    F = loads.table(load, time, model)
    s = cpu.NewmarkCPU(M, C, K, spec["dt"])
    return s, F, ForceTable.from_dense(F), time, (M, C, K)


def test_cpu_baseline_record():
    import bench

    s, _, table, _, _ = _system()
    rec = np.arange(0, s.n, 7)
    cb = bench.cpu_baseline_run(s.n, s.rowptr, s.cols, s.M, s.C, s.K, table, rec, target_s=0.5, max_steps=8)
    assert cb["kind"] == "port" and cb["unit"] == "DOF-steps/s"
    assert cb["value"] > 0 and cb["cores"] >= 1
    assert "iterations per step" in cb["sample"]


def test_cpu_loop_matches_direct_solve():
    from oracle import newmark

    s, F, table, time, (M, C, K) = _system()
    n_t = 200
    out, iters = s.run(0, n_t - 1, table.f_ptr, table.f_eq, table.f_val, np.arange(s.n))
    U, V, A, _ = newmark.solve(M, C, K, F[:n_t], time[:n_t], 1)
    assert iters > 0
    assert rel_l2(out, V[1:n_t]) <= 1e-10
