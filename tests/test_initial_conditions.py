"""Initial conditions in the reference solver's duck type: u[0, :] and v[0, :] are writable
after initialise() and calculate() starts from them.  This checks the host side with a test
double for the device solver: the state reaches it before the initial acceleration, a start
from rest sends none, and the explicit scheme (rest only) refuses other initial conditions."""
from types import SimpleNamespace

import numpy as np
import pytest
import scipy.sparse as sp


class FakeDeviceSolver:
    """Records the calls NewmarkExplicit.calculate makes on a device solver."""

    made = []

    def __init__(self, *args, **kwargs):
        self.calls = []
        FakeDeviceSolver.made.append(self)

    def set_force(self, table, stream=False):
        self.calls.append("set_force")

    def push_force(self, t_begin, t_end):
        pass

    def set_output(self, interval, rec, n_out, what=("u", "v", "a")):
        self.n_out, self.n_rec = n_out, len(rec)
        self.calls.append("set_output")

    def set_state(self, u0, v0):
        self.calls.append(("set_state", np.array(u0), np.array(v0)))

    def initial_acceleration(self):
        self.calls.append("initial_acceleration")

    def run(self, t_begin, t_end):
        self.calls.append(("run", t_begin, t_end))

    def status(self):
        return 0, 0, 0

    def output_rows(self, r0, r1):
        z = np.zeros((r1 - r0 + 1, self.n_rec))
        return {"u": z, "v": z, "a": z}

    def close(self):
        pass


def _run(monkeypatch, u0, v0):
    from scatter_gb300 import solvers

    monkeypatch.setattr(solvers, "_device_matrices", lambda M, C, K: (SimpleNamespace(n=M.shape[0]), None, None, None))
    monkeypatch.setattr(solvers, "NewmarkGPU", FakeDeviceSolver)
    n, time = len(u0), np.arange(5) * 1e-3
    M = sp.identity(n, format="csr")
    s = solvers.NewmarkExplicit(layout="csr")
    s.initialise(n, time)
    s.u[0], s.v[0] = u0, v0
    s.update(0)
    s.calculate(M, M, M, np.zeros(n), 0, len(time) - 1)
    return FakeDeviceSolver.made[-1].calls


def test_initial_state_reaches_the_device_solver(monkeypatch):
    u0 = np.linspace(0.0, 1e-3, 6)
    v0 = -np.linspace(0.0, 2e-2, 6)
    calls = _run(monkeypatch, u0, v0)
    states = [c for c in calls if isinstance(c, tuple) and c[0] == "set_state"]
    assert len(states) == 1
    np.testing.assert_array_equal(states[0][1], u0)
    np.testing.assert_array_equal(states[0][2], v0)
    # before the initial acceleration, which then solves M a0 = f(0) - C v0 - K u0
    assert calls.index(states[0]) + 1 == calls.index("initial_acceleration")
    assert calls[-1] == ("run", 0, 4)


def test_start_from_rest_sends_no_state(monkeypatch):
    calls = _run(monkeypatch, np.zeros(6), np.zeros(6))
    assert not any(isinstance(c, tuple) and c[0] == "set_state" for c in calls)
    assert "initial_acceleration" in calls


def test_explicit_scheme_refuses_initial_conditions(monkeypatch):
    from scatter_gb300 import explicit

    class Assembled:  # stands in for the GenerateMatrix the scheme requires
        pass

    monkeypatch.setattr(explicit, "GenerateMatrix", Assembled)
    s = explicit.ExplicitLumped()
    s.initialise(6, np.arange(5) * 1e-4)
    s.v[0, 3] = 0.1
    g = Assembled()
    with pytest.raises(NotImplementedError, match="starts from rest"):
        s.calculate(g, g, g, None, 0, 4)
