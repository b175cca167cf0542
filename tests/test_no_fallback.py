"""The product path has no CPU fallback: without a CUDA device the reference-facing entry
point and the solvers raise, and a missing CUDA library raises instead of being skipped.
(These run where no GPU is present; on a GPU machine the same calls are the GPU tests.)"""
import os
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from helpers import case, oracle_system

no_gpu = pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a CUDA device")


def _gmsh(name, tmp_path):
    from scatter_gb300 import meshgen

    model, spec = case(name)
    dim = int(model["dimension"])
    src = SimpleNamespace(nodes=model["nodes"], elem=model["elem"], element_type=model["element_type"],
                          materials=[[dim, int(i), str(n)] for i, n in zip(model["material_ids"],
                                                                           model["material_names"])],
                          materials_index=model["materials_index"])
    path = os.path.join(tmp_path, f"{name}.msh")
    meshgen.write_gmsh(path, src)
    return path, spec


@no_gpu
def test_scatter_entry_point_raises_without_gpu(tmp_path):
    from scatter_gb300.scatter import scatter

    path, spec = _gmsh("column_hexa8_pulse", tmp_path)
    settings = {"int_order": 2, "damping": spec["damping"], "absorbing_BC": spec["absorbing"],
                "absorbing_BC_stiff": spec["k_div"], "pickle": True, "pickle_nodes": "all", "VTK": False,
                "VTK_binary": True}
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        scatter(path, str(tmp_path / "out"), spec["materials"], spec["boundaries"], settings, dict(spec["load"]),
                time_step=spec["dt"])
    assert not (tmp_path / "out" / "data.pickle").exists()


@no_gpu
def test_solver_on_scipy_matrices_raises_without_gpu():
    from scatter_gb300.solvers import NewmarkExplicit

    model, spec, M, C, K, _, _ = oracle_system("tetra4_bench2")
    time = np.arange(5) * spec["dt"]
    s = NewmarkExplicit(layout="csr")
    s.initialise(M.shape[0], time)
    s.update(0)
    with pytest.raises(RuntimeError, match="no CPU fallback|CUDA"):
        s.calculate(M, C, K, np.zeros(M.shape[0]), 0, len(time) - 1)


def test_missing_library_raises(monkeypatch, tmp_path):
    from scatter_gb300 import _native

    monkeypatch.setattr(_native, "_lib", None)
    monkeypatch.setattr(_native._build, "LIB", str(tmp_path / "absent.so"))
    with pytest.raises(RuntimeError, match="not built"):
        _native.load()
