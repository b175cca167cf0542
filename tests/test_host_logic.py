"""Host-side logic of the GPU path (no GPU): mesh reading and numbering, Lysmer face
ordering, force tables -- each against the reference's golden vectors."""
import os
from types import SimpleNamespace

import numpy as np
import pytest
import scipy.sparse as sp

from helpers import case, golden_csr, golden_load_table, npz
from scatter_gb300 import meshgen
from scatter_gb300.mesher import ReadMesh

CASES = ["column_hexa8_pulse", "column_hexa8_abs", "column_hexa20_abs", "quad4_2d", "tri3_bench2", "tri6_bench2",
         "tetra4_bench2", "tetra10_bench2", "tetra10_abs", "cube_abs5", "cube_moving"]


def _read_back(name, tmp_path):
    model, spec = case(name)
    dim = int(model["dimension"])
    src = SimpleNamespace(nodes=model["nodes"], elem=model["elem"], element_type=model["element_type"],
                          materials=[[dim, int(i), str(n)] for i, n in zip(model["material_ids"], model["material_names"])],
                          materials_index=model["materials_index"])
    path = os.path.join(tmp_path, f"{name}.msh")
    meshgen.write_gmsh(path, src)
    m = ReadMesh(path)
    m.read_gmsh()
    m.read_bc(spec["boundaries"])
    m.mapping()
    m.connectivities()
    m.get_mesh_edges()
    return m, model, spec


@pytest.mark.parametrize("name", CASES)
def test_mesher_numbering(name, tmp_path):
    m, model, spec = _read_back(name, tmp_path)
    assert m.element_type == model["element_type"] and m.dimension == model["dimension"]
    np.testing.assert_array_equal(m.BC, model["BC"])
    np.testing.assert_array_equal(m.BC_dir, model["BC_dir"])
    np.testing.assert_array_equal(m.eq_nb_dof, model["eq_nb_dof"])
    np.testing.assert_array_equal(m.eq_nb_elem, model["eq_nb_elem"])
    assert m.number_eq == model["number_eq"]
    if "boundary_elem" in model:
        np.testing.assert_array_equal(m.boundary_elem, model["boundary_elem"])


@pytest.mark.parametrize("name", ["column_hexa8_abs", "column_hexa20_abs", "tetra4_abs", "tetra10_abs", "cube_abs5"])
def test_lysmer_face_ordering(name):
    """Host face ordering + oracle face integrals reproduce the reference's absorbing matrices."""
    from helpers import element_props
    from oracle import elements as el
    from scatter_gb300.lysmer import boundary_faces
    from scatter_gb300.system_matrix import FACE_TYPES

    model, spec = case(name)
    ns = SimpleNamespace(**{k: model[k] for k in ("nodes", "elem", "BC", "BC_dir", "eq_nb_dof")},
                         element_type=model["element_type"])
    props = element_props(model, spec["materials"])
    faces = boundary_faces(ns, props, spec["absorbing"])
    F = el.face_matrix(FACE_TYPES[model["element_type"]], faces["xy"], 2)
    n = model["number_eq"]
    nf = faces["eqs"].shape[1]
    r = np.repeat(faces["eqs"], nf, axis=1).ravel()
    c = np.tile(faces["eqs"], (1, nf)).ravel()
    Cv = (F * faces["fct"][:, None, :]).ravel()
    Kv = (np.abs(F) * faces["fct2"][:, None, :]).ravel()
    C = sp.csr_matrix((Cv, (r, c)), shape=(n, n))
    K = sp.csr_matrix((Kv, (r, c)), shape=(n, n)) / spec["k_div"]
    g = npz(f"mat_{name}.npz")
    gC, gK = golden_csr(g, "Cabs"), golden_csr(g, "Kabs")
    assert gC.nnz > 0
    assert abs(C - gC).max() <= 1e-14 * abs(gC).max()
    assert abs(K - gK).max() <= 1e-14 * abs(gK).max()


@pytest.mark.parametrize("name", ["column_hexa8_pulse", "column_hexa8_abs", "quad4_2d", "tri3_bench2",
                                  "tetra10_bench2", "cube_moving", "cube_plane"])
def test_force_tables(name, tmp_path):
    from scatter_gb300.force_external import Force
    from scatter_gb300.validator import ValidateLoad

    m, model, spec = _read_back(name, tmp_path)
    load = dict(spec["load"])
    ValidateLoad.validate(load)
    time = np.linspace(0, load["time"], int(np.ceil(load["time"] / spec["dt"]) + 1))
    top = m.get_top_surface() if load["type"] == "moving_at_plane" else []
    F = Force()
    F.initialise_load(load, time, m, None, top_surface_elements=top)
    Fg, tg = golden_load_table(name)
    dense = np.stack([F.table.dense(t) for t in range(len(time))])
    assert np.abs(dense - Fg).max() <= 1e-12 * max(np.abs(Fg).max(), 1.0)
    np.testing.assert_array_equal(F.update_load_at_t(3), Fg[3])


def test_structured_box_numbering_and_jacobian():
    from oracle import elements as el

    m = meshgen.box_model(3, 4, 2, 0.5, bottom="020", x_faces="200", z_faces="002")
    assert m.number_eq == 3 * len(m.nodes)
    X = m.nodes[:, 1:][m.elem - 1]
    _, _, detJ, _ = el.geometry("hexa8", X, 2)
    assert (detJ > 0).all()
    t = meshgen.box_model(2, 2, 2, 0.5, element="tetra10")
    X = t.nodes[:, 1:][t.elem - 1]
    _, _, detJ, _ = el.geometry("tetra10", X, 2)
    assert (detJ > 0).all()
    # conforming: every mid-side node is shared by all tets around its edge
    assert len(t.nodes) == (5 * 5 * 5)  # (2*2+1)^3 vertices + mid-sides on the refined lattice


def test_validator_defaults():
    from scatter_gb300.validator import ValidateLoad

    load = {"type": "heaviside"}
    ValidateLoad.validate(load)
    assert load["ini_steps"] == 5
    with pytest.raises(Exception):
        ValidateLoad.validate({"type": "unknown"})


def test_ragged_mesh_specs_seeded():
    from scatter_gb300.ragged import mesh_specs

    a = mesh_specs(64, seed=3)
    b = mesh_specs(64, seed=3)
    assert a == b and len(a) == 64
    assert {s["element"] for s in a} == {"hexa8", "tetra10"}
    for s in a:
        lo, hi = (10, 80) if s["element"] == "hexa8" else (5, 40)
        assert all(lo <= d <= hi for d in s["dims"])
        assert 20e6 <= s["E"] <= 200e6 and 0.2 <= s["nu"] <= 0.35 and 1700 <= s["rho"] <= 2100


def test_hrz_lumping_of_the_reference_tetra10_mass_is_positive():
    """Row sums of the reference's tetra10 consistent mass are negative at the corners, so the
    ragged path lumps quadratic tetrahedra by diagonal scaling; the oracle's HRZ mass is
    positive and keeps the element mass."""
    import numpy as np

    from oracle import elements as el
    from scatter_gb300 import meshgen

    m = meshgen.box_model(1, 1, 1, 0.5, element="tetra10")
    X = m.nodes[:, 1:][m.node_index()[m.elem]]
    n = len(m.elem)
    _, Me = el.element_matrices("tetra10", X, np.ones(n), np.full(n, 0.3), np.full(n, 2000.0))
    Mx = Me[0][::3, ::3]
    assert Mx.sum(axis=1)[:4].max() < 0  # corner row sums
    f = Mx.sum() / np.trace(Mx)
    lumped = f * np.diag(Mx)
    assert lumped.min() > 0
    assert abs(lumped.sum() / Mx.sum() - 1) < 1e-12


def test_matrix_free_lumped_mass_equals_assembled_row_sums():
    """The per-element lumped-mass contributions of the matrix-free ragged path (row sums over
    free columns, scattered to nodes) equal the row sums of the assembled consistent mass."""
    import numpy as np

    from oracle import assembly as asm
    from oracle import elements as el
    from oracle import explicit
    from scatter_gb300 import meshgen
    from scatter_gb300.system_matrix import model_arrays

    m = meshgen.box_model(3, 4, 2, 0.5, element="hexa8")
    nodes, _, elem_idx, eqmap = model_arrays(m)
    n = len(elem_idx)
    _, Me = el.element_matrices("hexa8", nodes[:, 1:][elem_idx], np.ones(n), np.full(n, 0.25), np.ones(n))
    from scatter_gb300.ragged import lumped_mass

    Mx = Me.reshape(n, 8, 3, 8, 3)[:, :, 0, :, 0]
    free = eqmap >= 0
    ml = lumped_mass(Mx, np.arange(n), elem_idx, free, 1.0)
    ref = explicit.lumped(asm.assemble(m.eq_nb_elem, Me, m.number_eq))
    nn, cc = np.nonzero(free)
    assert np.abs(ml[nn, cc] - ref[eqmap[nn, cc]]).max() <= 1e-14 * ref.max()
    # diagonal scaling keeps each element's mass
    mt = meshgen.box_model(1, 1, 1, 0.5, element="tetra10")
    nd_, _, ei, em = model_arrays(mt)
    k = len(ei)
    _, Mt = el.element_matrices("tetra10", nd_[:, 1:][ei], np.ones(k), np.full(k, 0.3), np.ones(k))
    Mtx = Mt.reshape(k, 10, 3, 10, 3)[:, :, 0, :, 0]
    h = lumped_mass(Mtx, np.arange(k), ei, np.ones_like(em, dtype=bool), 1.0, hrz=True)
    assert h.min() > 0 and abs(h[:, 0].sum() / Mtx.sum() - 1) < 1e-12


def test_batched_incidence_and_hex8_grid_tables():
    """Host tables of the batched step: incidence lists ordered by the node's local index in
    the element, and the uniform hexa8 grid tables (every element's node lb found in the tile
    halo of its node la at the natural offset between them), None for meshes that are not such
    grids."""
    from scatter_gb300.batched import HEX8_NAT, HEX8_TILE, hex8_grid_tables, incidence_by_local_index
    from scatter_gb300.system_matrix import model_arrays

    m = meshgen.box_model(5, 3, 4, 0.5)
    nodes, _, elem_idx, _ = model_arrays(m)
    xyz = nodes[:, 1:].astype(float)
    N, E = len(nodes), len(elem_idx)
    ptr, inc = incidence_by_local_index(elem_idx, N)
    assert ptr[-1] == E * 8
    for a in (0, N // 2, N - 1):
        els = inc[ptr[a]:ptr[a + 1]]
        las = [int(np.nonzero(elem_idx[e] == a)[0][0]) for e in els]
        assert las == sorted(las) and sorted(els.tolist()) == sorted(np.nonzero((elem_idx == a).any(1))[0].tolist())
    halo, elem8 = hex8_grid_tables(xyz, elem_idx)
    tx, ty, tz = HEX8_TILE
    hx, hy = tx + 2, ty + 2
    assert halo.shape[1] == hx * hy * (tz + 2)
    # each node owned by exactly one tile (the halo's interior points)
    inner = [(x + 1) + hx * ((y + 1) + hy * (z + 1)) for z in range(tz) for y in range(ty) for x in range(tx)]
    owned = halo[:, inner].ravel()
    owned = owned[owned >= 0]
    assert len(owned) == N and len(np.unique(owned)) == N
    where = {}
    for t in range(len(halo)):
        for p in inner:
            if halo[t, p] >= 0:
                where[int(halo[t, p])] = (t, p)
    for e in range(E):
        for la in range(8):
            a = elem_idx[e, la]
            assert elem8[a, la] == e
            t, p = where[int(a)]
            for lb in range(8):
                d = HEX8_NAT[lb] - HEX8_NAT[la]
                assert halo[t, p + d[0] + hx * (d[1] + hy * d[2])] == elem_idx[e, lb]
    # boundary: a corner node has one element; its halo holds -1 outside the mesh
    deg = np.bincount(elem_idx.ravel(), minlength=N)
    corner = int(np.nonzero(deg == 1)[0][0])
    assert (elem8[corner] >= 0).sum() == 1
    assert (halo == -1).any()
    # a reversed element breaks the common orientation
    bad = elem_idx.copy()
    bad[3] = bad[3][[1, 0, 3, 2, 5, 4, 7, 6]]
    assert hex8_grid_tables(xyz, bad) is None


def test_hex8_grid_tables_with_holes():
    """An L-shaped structured hexa8 mesh (a box with one quarter removed): every element's
    nodes are found in the tile halos at their natural offsets, the removed quarter's lattice
    points are -1 in the halos, and every node is owned by exactly one tile."""
    from scatter_gb300.batched import HEX8_NAT, HEX8_TILE, hex8_grid_tables
    from scatter_gb300.system_matrix import model_arrays

    m = meshgen.box_model(9, 3, 7, 0.5)
    nodes, _, elem_idx, _ = model_arrays(m)
    xyz = nodes[:, 1:].astype(float)
    c = xyz[elem_idx].mean(axis=1)
    keep = ~((c[:, 0] > 2.0) & (c[:, 2] < c[:, 2].min() + 1.5))  # drop a corner block of elements
    el = elem_idx[keep]
    used = np.unique(el)
    remap = -np.ones(len(xyz), dtype=np.int64)
    remap[used] = np.arange(len(used))
    el = remap[el]
    xyz = xyz[used]
    N, E = len(xyz), len(el)
    halo, elem8 = hex8_grid_tables(xyz, el)
    tx, ty, tz = HEX8_TILE
    hx, hy = tx + 2, ty + 2
    inner = [(x + 1) + hx * ((y + 1) + hy * (z + 1)) for z in range(tz) for y in range(ty) for x in range(tx)]
    owned = halo[:, inner].ravel()
    owned = owned[owned >= 0]
    assert len(owned) == N and len(np.unique(owned)) == N
    assert (halo[:, inner] == -1).any()  # lattice points of the removed block
    where = {}
    for t in range(len(halo)):
        for p in inner:
            if halo[t, p] >= 0:
                where[int(halo[t, p])] = (t, p)
    for e in range(E):
        for la in range(8):
            a = el[e, la]
            assert elem8[a, la] == e
            t, p = where[int(a)]
            for lb in range(8):
                d = HEX8_NAT[lb] - HEX8_NAT[la]
                assert halo[t, p + d[0] + hx * (d[1] + hy * d[2])] == el[e, lb]
    # nodes at the re-entrant corner have fewer than 8 elements
    assert ((elem8 >= 0).sum(axis=1) < 8).sum() > 0


def _replay_column_kernel(tables, elem_idx, Ke, w, seg):
    """The tensor-core step's decomposition replayed on the CPU: per column and segment, the
    element layers kbeg .. kend - 1, each element position's forces Ke w added to the owned
    points of planes k and k + 1, plane k kept after layer k when it is in the segment, and the
    top plane kept after the last layer.  Returns the forces [n_nodes, 3] and how many times
    each node was finished."""
    from scatter_gb300.batched import HEX8_COLUMN, HEX8_NAT

    nodes, elems, nzp = tables
    cx, cy = HEX8_COLUMN
    chx = cx + 2
    f = np.zeros((len(w), 3))
    done = np.zeros(len(w), dtype=int)
    n_segs = -(-nzp // seg)
    for col in range(len(nodes)):
        for sg in range(n_segs):
            z0, z1 = sg * seg, min(sg * seg + seg, nzp)
            kbeg, kend = max(z0 - 1, 0), min(z1, nzp - 1)
            cur, nxt = np.zeros((cx * cy, 3)), np.zeros((cx * cy, 3))

            def finish(plane, acc):
                for p in range(cx * cy):
                    a = nodes[col, plane, (p // cx + 1) * chx + p % cx + 1]
                    if a >= 0:
                        f[a] += acc[p]
                        done[a] += 1

            for k in range(kbeg, kend):
                for P in range((cx + 1) * (cy + 1)):
                    e = elems[col, k, P]
                    if e < 0:
                        continue
                    ex, ey = P % (cx + 1), P // (cx + 1)
                    ring = [nodes[col, k + HEX8_NAT[l, 2], (ey + HEX8_NAT[l, 1]) * chx + ex + HEX8_NAT[l, 0]]
                            for l in range(8)]
                    assert ring == list(elem_idx[e])
                    d = Ke[e] @ w[elem_idx[e]].ravel()
                    for l in range(8):
                        hx, hy = ex + HEX8_NAT[l, 0], ey + HEX8_NAT[l, 1]
                        if 1 <= hx <= cx and 1 <= hy <= cy:
                            (cur if HEX8_NAT[l, 2] == 0 else nxt)[(hy - 1) * cx + hx - 1] += d[3 * l:3 * l + 3]
                if k >= z0:
                    finish(k, cur)
                cur, nxt = nxt, np.zeros((cx * cy, 3))
            if kend < z1:
                finish(kend, cur)
    return f, done


@pytest.mark.parametrize("notched", [False, True])
def test_hex8_column_tables_cover_every_element_once(notched):
    """The tensor-core step's column tables and decomposition: on a box and on an L-shaped box,
    every node is finished exactly once per step for every segment length, and the forces it
    gathers equal the assembled K w."""
    from oracle import assembly as asm
    from oracle import elements as el
    from scatter_gb300.batched import hex8_column_tables
    from scatter_gb300.system_matrix import model_arrays

    m = meshgen.box_model(9, 5, 6, 0.5)
    nodes, _, elem_idx, _ = model_arrays(m)
    xyz = nodes[:, 1:].astype(float)
    if notched:
        c = xyz[elem_idx].mean(axis=1)
        keep = ~((c[:, 0] > 2.0) & (c[:, 2] < c[:, 2].min() + 1.5))
        el_k = elem_idx[keep]
        used = np.unique(el_k)
        remap = -np.ones(len(xyz), dtype=np.int64)
        remap[used] = np.arange(len(used))
        elem_idx, xyz = remap[el_k], xyz[used]
    tables = hex8_column_tables(xyz, elem_idx)
    assert tables is not None
    N, E = len(xyz), len(elem_idx)
    rng = np.random.default_rng(0)
    Ke, _ = el.element_matrices("hexa8", xyz[elem_idx], rng.uniform(1, 2, E), np.full(E, 0.3), np.ones(E))
    eq = np.arange(3 * N, dtype=float).reshape(N, 3)
    K = asm.assemble(eq[elem_idx].reshape(E, 24), Ke, 3 * N)
    w = rng.standard_normal((N, 3))
    want = (K @ w.ravel()).reshape(N, 3)
    for seg in sorted({tables[2], -(-tables[2] // 2), 3, 1}):
        f, done = _replay_column_kernel(tables, elem_idx, Ke, w, seg)
        assert np.all(done == 1), seg
        np.testing.assert_allclose(f, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
    bad = elem_idx.copy()
    bad[3] = bad[3][[1, 0, 3, 2, 5, 4, 7, 6]]
    assert hex8_column_tables(xyz, bad) is None
