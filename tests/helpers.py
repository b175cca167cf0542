"""Shared test helpers: load golden fixtures, build oracle inputs."""
import ast
import os

import numpy as np
import scipy.sparse as sp

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def npz(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def case(name):
    """Model dict (the reference's ReadMesh output) and the case settings."""
    d = npz(f"mesh_{name}.npz")
    model = {k: d[k] for k in d.files if not k.startswith("case_")}
    model["element_type"] = str(model["element_type"])
    model["number_eq"] = int(model["number_eq"])
    model["dimension"] = int(model["dimension"])
    spec = {k[5:]: ast.literal_eval(str(d[k])) for k in d.files if k.startswith("case_")}
    return model, spec


def element_props(model, materials):
    """Per-element (E, nu, rho) through the physical-group names (system_matrix.py:64-71)."""
    names = dict(zip(model["material_ids"].tolist(), model["material_names"].tolist()))
    mi = model["materials_index"]
    E = np.array([materials[names[int(i)]]["Young"] for i in mi], dtype=float)
    nu = np.array([materials[names[int(i)]]["poisson"] for i in mi], dtype=float)
    rho = np.array([materials[names[int(i)]]["density"] for i in mi], dtype=float)
    return E, nu, rho


def element_coords(model):
    nodes = model["nodes"]
    id2idx = np.zeros(int(nodes[:, 0].max()) + 1, dtype=np.int64)
    id2idx[nodes[:, 0].astype(np.int64)] = np.arange(len(nodes))
    return nodes[id2idx[model["elem"]], 1:]


def golden_csr(mats, prefix):
    if prefix + "_data" not in mats.files:
        return None
    shape = tuple(mats[prefix + "_shape"])
    return sp.csr_matrix((mats[prefix + "_data"], mats[prefix + "_indices"], mats[prefix + "_indptr"]), shape=shape)


def pattern_hash(a):
    import hashlib

    a = sp.csr_matrix(a)
    a.sort_indices()
    h = hashlib.sha256()
    h.update(np.asarray(a.indptr, dtype=np.int64).tobytes())
    h.update(np.asarray(a.indices, dtype=np.int64).tobytes())
    return h.hexdigest()


def golden_load_table(name, n_t=None):
    d = npz(f"load_{name}.npz")
    n = int(d["n_eq"])
    T = len(d["time"]) if n_t is None else n_t
    F = np.zeros((T, n))
    sel = d["step"] < T
    F[d["step"][sel], d["eq"][sel]] = d["val"][sel]
    return F, d["time"]


def rel_l2(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def model_ns(name):
    """A ReadMesh-like object from the golden mesh fixture (for the GPU GenerateMatrix)."""
    from types import SimpleNamespace

    model, spec = case(name)
    ns = SimpleNamespace(
        nodes=model["nodes"], elem=model["elem"], materials_index=model["materials_index"],
        materials=[[0, int(i), str(n)] for i, n in zip(model["material_ids"], model["material_names"])],
        element_type=model["element_type"], dimension=model["dimension"], eq_nb_dof=model["eq_nb_dof"],
        eq_nb_elem=model["eq_nb_elem"], BC=model["BC"], BC_dir=model["BC_dir"], number_eq=model["number_eq"])
    return ns, model, spec


def oracle_system(name):
    """Oracle K, M, C (scipy CSR) for a golden case (reference semantics incl. zero dropping)."""
    from oracle import assembly as asm
    from oracle import elements as el
    from oracle import lysmer

    model, spec = case(name)
    E, nu, rho = element_props(model, spec["materials"])
    xyz = element_coords(model)
    Ke, Me = el.element_matrices(model["element_type"], xyz, E, nu, rho)
    pairs = asm.element_pairs(model["eq_nb_elem"])
    K0 = asm.assemble(model["eq_nb_elem"], Ke, model["number_eq"], pairs)
    M = asm.assemble(model["eq_nb_elem"], Me, model["number_eq"], pairs)
    Ca, Ka = lysmer.absorbing(model, (E, nu, rho), spec["absorbing"], spec["k_div"])
    K = asm.drop_zeros(K0 + Ka)
    C = asm.rayleigh(M, K, Ca, spec["damping"])
    return model, spec, M, C, K, Ca, Ka


def full_field(X, eq_nb_dof):
    """[n_t, n_eq] equation results -> [n_t, n_nodes, dim] with zeros at fixed DOFs
    (export_results.py:85-97)."""
    eq = np.asarray(eq_nb_dof, dtype=float)
    out = np.zeros((X.shape[0], eq.shape[0], eq.shape[1]))
    for c in range(eq.shape[1]):
        m = ~np.isnan(eq[:, c])
        out[:, m, c] = X[:, eq[m, c].astype(int)]
    return out
