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
    cb, v = bench.cpu_baseline_run(s.n, s.rowptr, s.cols, s.M, s.C, s.K, table, rec, target_s=0.5, max_steps=8,
                                   dt=s.dt)
    assert cb["kind"] == "port" and cb["unit"] == "DOF-steps/s"
    assert cb["value"] > 0 and cb["cores"] >= 1
    assert "iterations per step" in cb["sample"]
    # receiver velocities after steps 1 .. steps + 1, from rest: the history the bench checks
    # the GPU loop against
    from oracle import newmark

    _, F, _, time, (M, C, K) = _system()
    V = newmark.solve(M, C, K, F[:len(v) + 1], time[:len(v) + 1], 1)[1]
    assert rel_l2(v, V[1:, rec]) <= 1e-10
    p = bench.parity_record(V[1:, rec] * (1 + 1e-12), v)
    assert p["ok"] and p["steps"] == len(v)
    assert not bench.parity_record(V[1:, rec] * (1 + 1e-6), v)["ok"]


def test_cpu_loop_matches_direct_solve():
    from oracle import newmark

    s, F, table, time, (M, C, K) = _system()
    n_t = 200
    out, iters = s.run(0, n_t - 1, table.f_ptr, table.f_eq, table.f_val, np.arange(s.n))
    U, V, A, _ = newmark.solve(M, C, K, F[:n_t], time[:n_t], 1)
    assert iters > 0
    assert rel_l2(out, V[1:n_t]) <= 1e-10
