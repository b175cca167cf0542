"""Entry point with the reference's signature and dictionaries (scatter/scatter.py:36-171).

    from scatter_gb300.scatter import scatter, Solver
    res = scatter(mesh_file, out_folder, materials, boundaries, inp_settings, loading,
                  time_step=5e-4, solver=Solver.NEWMARK_EXPLICIT)

Element integration, assembly, Lysmer boundaries, Rayleigh damping and the time loop run on
the GPU; mesh reading, equation numbering, load tabulation and export stay on the host.
``solver`` takes the reference's Solver members; NEWMARK_EXPLICIT (the reference default,
numerically the average-acceleration Newmark) runs on the GPU.  EXPLICIT_LUMPED is the
added matrix-free central-difference scheme (lumped mass), which has no reference
counterpart.  The other members belong to the external PuggleSolvers package and raise.
"""
import numpy as np

from . import export_results, force_external, mesher, system_matrix, validator
from .solvers import NewmarkExplicit


class Solver:
    """The reference's Solver enum values (scatter/scatter.py:16-33) plus the GPU-only scheme."""

    STATIC = "StaticSolver"
    NEWMARK_EXPLICIT = "NewmarkExplicit"
    NEWMARK_IMPLICIT = "NewmarkImplicitForce"
    CENTRAL_DIFFERENCE = "CentralDifferenceSolver"
    BATHE = "BatheSolver"
    EXPLICIT_LUMPED = "ExplicitLumpedGPU"


def _solver_value(solver):
    return getattr(solver, "value", solver)


def scatter(mesh_file, outfile_folder, materials, boundaries, inp_settings, loading, time_step=0.1,
            solver=Solver.NEWMARK_EXPLICIT, random_props=False, receivers=None):
    """Run the wave-propagation model on the GPU; returns an export_results.Write."""
    validator.ValidateLoad.validate(loading)
    model = mesher.ReadMesh(mesh_file)
    model.read_gmsh()
    model.read_bc(boundaries)
    model.mapping()
    model.connectivities()
    if loading["type"] == "rose":
        raise NotImplementedError("ROSE train-track coupling is outside this GPU path")
    model.get_mesh_edges()
    if random_props:
        from .random_fields import RF

        rf = RF(random_props, materials, outfile_folder, model.element_type)
        mat_idx = [m[1] for m in model.materials if m[2] == random_props["material"]][0]
        elements = model.elem[model.materials_index == mat_idx]
        rf.generate_gstools_rf(model.nodes, elements, model.dimension, angles=0.0)
        rf.dump()
        rf.update_material_list(materials, model, mat_idx)
        materials.update(rf.new_material)

    matrix = system_matrix.GenerateMatrix(model.number_eq, inp_settings["int_order"])
    matrix.generate_stiffness_and_mass(model, materials)
    matrix.absorbing_boundaries(model, materials, inp_settings["absorbing_BC"], inp_settings["absorbing_BC_stiff"])
    matrix.damping_Rayleigh(inp_settings["damping"])

    time = np.linspace(0, loading["time"], int(np.ceil(loading["time"] / time_step) + 1))
    kind = _solver_value(solver)
    if kind == Solver.NEWMARK_EXPLICIT:
        numerical = NewmarkExplicit()
    elif kind == Solver.EXPLICIT_LUMPED:
        from .explicit import ExplicitLumped

        numerical = ExplicitLumped()
    else:
        raise NotImplementedError(f"solver {kind} is not part of the GPU path (PuggleSolvers only)")
    numerical.output_interval = inp_settings.get("output_interval", 1)
    numerical.initialise(model.number_eq, time)

    F = force_external.Force()
    top = model.get_top_surface() if loading["type"] == "moving_at_plane" else []
    F.initialise_load(loading, time, model, numerical, top_surface_elements=top)
    numerical.update_rhs_at_time_step_func = F.update_load_at_t
    numerical.force_table = F.table
    if receivers is not None:
        numerical.receivers = receivers

    numerical.update(0)
    numerical.calculate(matrix, matrix, matrix, F.force_vector, 0, len(time) - 1)

    results = export_results.Write(outfile_folder, model, materials, numerical)
    results.pickle(write=inp_settings["pickle"], nodes=inp_settings["pickle_nodes"])
    results.vtk(write=inp_settings["VTK"], binary=inp_settings["VTK_binary"], output_interval=1)
    return results
