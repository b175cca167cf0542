"""The reference-facing entry point scatter() end to end on CPU.

The two GPU stages (GenerateMatrix and the device time loop) are replaced by test doubles that
compute with the oracle.  Everything else is the entry point's own code: the load validator,
the gmsh reader and equation numbering, the force table, the solver set-up and the export.
The checker is the reference's golden history for its benchmark set 2
(integration_tests/test_benchmark_set_2.py), read back from the pickle scatter() writes."""
import os
import pickle
from types import SimpleNamespace

import numpy as np

from helpers import case, element_coords, element_props, npz, rel_l2


def _as_dict(model):
    mats = model.materials
    return {"nodes": np.asarray(model.nodes), "elem": np.asarray(model.elem), "eq_nb_elem": model.eq_nb_elem,
            "eq_nb_dof": model.eq_nb_dof, "BC": model.BC, "BC_dir": model.BC_dir,
            "element_type": model.element_type, "number_eq": int(model.number_eq),
            "materials_index": np.asarray(model.materials_index),
            "material_ids": np.array([int(m[1]) for m in mats]), "material_names": np.array([m[2] for m in mats])}


class OracleMatrix:
    """Stands in for system_matrix.GenerateMatrix (same calls), assembling with the oracle."""

    def __init__(self, number_eq, int_order):
        self.number_eq, self.order = number_eq, int_order

    def generate_stiffness_and_mass(self, model, materials):
        from oracle import assembly as asm
        from oracle import elements as el

        self.model = _as_dict(model)
        self.props = element_props(self.model, materials)
        Ke, Me = el.element_matrices(self.model["element_type"], element_coords(self.model), *self.props,
                                     order=self.order)
        pairs = asm.element_pairs(self.model["eq_nb_elem"])
        self.K0 = asm.assemble(self.model["eq_nb_elem"], Ke, self.number_eq, pairs)
        self.M = asm.assemble(self.model["eq_nb_elem"], Me, self.number_eq, pairs)

    def absorbing_boundaries(self, model, materials, absorbing, k_div):
        from oracle import assembly as asm
        from oracle import lysmer

        self.Ca, Ka = lysmer.absorbing(self.model, self.props, absorbing, k_div)
        self.K = asm.drop_zeros(self.K0 + Ka)

    def damping_Rayleigh(self, damping):
        from oracle import assembly as asm

        self.C = asm.rayleigh(self.M, self.K, self.Ca, damping)


class OracleNewmark:
    """Stands in for solvers.NewmarkExplicit (same attributes and calls), solving with the
    oracle's Newmark restatement over the force table scatter() hands it."""

    def __init__(self):
        self.output_interval = 1
        self.update_rhs_at_time_step_func = None
        self.force_table = None
        self.receivers = None
        self.calls = []

    def initialise(self, number_equations, time):
        self.number_equations = int(number_equations)
        self.time = np.asarray(time, dtype=float)
        self.output_time = self.time[::self.output_interval]

    def update(self, t_idx):
        self.calls.append(("update", t_idx))

    def calculate(self, M, C, K, F, t_start_idx, t_end_idx):
        from oracle import newmark

        self.calls.append(("calculate", t_start_idx, t_end_idx))
        assert M is C is K  # the entry point hands over the assembled object itself
        assert np.array_equal(F, self.force_table.dense(0))
        Fd = np.stack([self.force_table.dense(t) for t in range(len(self.time))])
        self.u, self.v, self.a, _ = newmark.solve(M.M, M.C, M.K, Fd, self.time, self.output_interval)


def test_scatter_entry_point_against_benchmark_set_2(tmp_path, monkeypatch):
    from scatter_gb300 import meshgen, system_matrix
    from scatter_gb300 import scatter as entry

    model, spec = case("tri3_bench2")
    dim = int(model["dimension"])
    src = SimpleNamespace(nodes=model["nodes"], elem=model["elem"], element_type=model["element_type"],
                          materials=[[dim, int(i), str(n)] for i, n in zip(model["material_ids"],
                                                                           model["material_names"])],
                          materials_index=model["materials_index"])
    mesh = os.path.join(tmp_path, "column_2D_tri3.msh")
    meshgen.write_gmsh(mesh, src)

    solvers = []

    def make_solver():
        solvers.append(OracleNewmark())
        return solvers[-1]

    monkeypatch.setattr(system_matrix, "GenerateMatrix", OracleMatrix)
    monkeypatch.setattr(entry, "NewmarkExplicit", make_solver)
    # the settings dictionary of the reference's integration tests
    settings = {"gamma": 0.5, "beta": 0.25, "int_order": 2, "damping": spec["damping"],
                "absorbing_BC": spec["absorbing"], "absorbing_BC_stiff": spec["k_div"], "pickle": True,
                "pickle_nodes": "all", "VTK": False, "VTK_binary": True}
    out = os.path.join(tmp_path, "results")
    res = entry.scatter(mesh, out, spec["materials"], spec["boundaries"], settings, dict(spec["load"]),
                        time_step=spec["dt"])

    s = solvers[0]
    assert s.calls[0] == ("update", 0) and s.calls[1][0] == "calculate"
    assert s.calls[1][1:] == (0, len(s.time) - 1)
    assert res.output_folder == out
    with open(os.path.join(out, "data.pickle"), "rb") as f:
        d = pickle.load(f)
    h = npz("hist_tri3_bench2.npz")
    assert len(d["time"]) == len(h["dis_y"])
    assert rel_l2(d["displacement"]["3"]["y"], h["dis_y"]) <= 1e-10
    assert rel_l2(d["velocity"]["3"]["y"], h["vel_y"]) <= 1e-10
    assert not os.path.exists(os.path.join(out, "VTK"))
