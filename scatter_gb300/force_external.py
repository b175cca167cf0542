"""External load as a device-ready force table: drop-in for scatter/force_external.py ``Force``.

The reference rebuilds a dense force vector every step in Python
(Force.update_load_at_t, force_external.py:55-74).  Here ``initialise_load`` tabulates the
whole history once as a :class:`ForceTable` (CSR over time) that the GPU step loop reads;
``update_load_at_t`` still returns the dense vector for callers that want it.

Load types and their reference semantics (kept for parity):
  pulse      triangular ramp over ini_steps, active while t < ini_steps - 1 (:76-84, :250-266)
  heaviside  linear ramp over ini_steps then 1 (:86-96, :268-279)
  moving     node line along z, two-node weights [1 - x/l, x*l] as written (:98-149, :320-345)
  moving_at_plane  point load on the hexa8 top surface, inverse-distance weights per axis,
             indicator weights when a node is within 1e-10 (:151-211, :281-318)
"""
import numpy as np
from scipy.spatial import cKDTree

from .solvers import ForceTable


def _ramp(n_t, steps):
    if n_t <= steps:
        raise SystemExit("Error: Number of loading steps smaller than " + str(steps))
    f = np.ones(n_t)
    f[:steps] = np.linspace(0, 1, steps)
    return f


class Force:
    def __init__(self):
        self.force_vector = []
        self.table = None

    def initialise_load(self, load_set, time, model, solver, **kwargs):
        self.nb_equations = int(model.number_eq)
        self.factor = load_set.get("force")
        self.contact_nodes = load_set.get("node")
        self.time = np.asarray(time, dtype=float)
        self.steps = load_set["ini_steps"]
        self.loading_type = load_set["type"]
        n_t = len(self.time)
        ids = np.asarray(model.nodes)[:, 0].astype(np.int64)
        id2idx = np.full(int(ids.max()) + 1, -1, dtype=np.int64)
        id2idx[ids] = np.arange(len(ids))
        eqmap = np.asarray(model.eq_nb_dof, dtype=float)
        kind = self.loading_type
        if kind in ("pulse", "heaviside"):
            if kind == "pulse":
                if n_t <= self.steps:
                    raise SystemExit("Error: Number of loading steps smaller than " + str(self.steps))
                sf = np.append(np.linspace(0, 1, int((self.steps - 1) / 2), endpoint=False),
                               np.linspace(1, 0, int((self.steps + 1) / 2)))
                active = np.arange(n_t) < self.steps - 1
            else:
                sf = _ramp(n_t, self.steps)
                active = np.ones(n_t, dtype=bool)
            # the dense vector is assigned node by node: the last assignment of an eq wins
            last = {}
            for n in self.contact_nodes:
                for i, eq in enumerate(eqmap[id2idx[int(n)]]):
                    if not np.isnan(eq):
                        last[int(eq)] = float(self.factor[i])
            eqs = np.array(sorted(last), dtype=np.int64)
            vals = np.array([last[e] for e in eqs])
            steps = np.nonzero(active)[0]
            counts = np.zeros(n_t, dtype=np.int64)
            counts[steps] = len(eqs)
            ptr = np.r_[0, np.cumsum(counts)]
            f_eq = np.tile(eqs, len(steps))
            f_val = (vals[None, :] * sf[steps][:, None]).ravel()
            self.table = _table_dropping_zeros(ptr, f_eq, f_val, self.nb_equations)
        elif kind == "moving":
            self.table = self._moving(load_set, model, id2idx, eqmap)
        elif kind == "moving_at_plane":
            self.table = self._moving_at_plane(load_set, model, id2idx, eqmap, kwargs["top_surface_elements"])
        elif kind == "rose":
            raise NotImplementedError("ROSE train-track loading is outside this GPU path")
        else:
            raise SystemExit(f'Error: Load type {load_set["type"]} not supported')
        self.force_vector = self.table.dense(0)

    def update_load_at_t(self, t, **kwargs):
        self.force_vector = self.table.dense(t)
        return self.force_vector

    # ------------------------------------------------------------------ moving (node line)
    def _moving(self, load, model, id2idx, eqmap):
        n_t = len(self.time)
        sf = _ramp(n_t, self.steps)
        nodes = np.asarray(model.nodes, dtype=float)
        idx = int(np.where(nodes[:, 0] == load["node"])[0][0]) if np.ndim(load["node"]) == 0 else \
            int(np.where(nodes[:, 0] == load["node"][0])[0][0])
        lst = np.where((nodes[:, 1] == nodes[idx, 1]) & (nodes[:, 2] == nodes[idx, 2]))[0]
        dist = np.sqrt((nodes[lst, 3] - nodes[idx, 3]) ** 2)
        lst = lst[np.argsort(dist)]
        dist = np.sort(dist)
        speed = np.ones(n_t) * load["speed"]
        speed[:self.steps] = 0
        ld = speed * (self.time - self.time[self.steps])
        ptr, eqs, vals = [0], [], []
        for t in range(n_t):
            entry = {}
            if ld[t] < np.max(dist):
                idn = np.where(dist <= ld[t])[0][-1]
                x = ld[t] - nodes[lst[idn], 3] + nodes[lst[0], 3]
                length = dist[idn + 1] - dist[idn]
                shp = np.array([1 - x / length, x * length])
                for j, ni in enumerate((lst[idn], lst[idn + 1])):
                    for i, eq in enumerate(eqmap[ni]):
                        if not np.isnan(eq):
                            entry[int(eq)] = float(self.factor[i]) * shp[j] * sf[t]
            ks = sorted(entry)
            eqs.extend(ks)
            vals.extend(entry[k] for k in ks)
            ptr.append(len(eqs))
        return _table_dropping_zeros(ptr, eqs, vals, self.nb_equations)

    # ------------------------------------------------------------------ moving at plane
    def _moving_at_plane(self, load, model, id2idx, eqmap, top):
        n_t = len(self.time)
        sf = _ramp(n_t, self.steps)
        X = np.asarray(model.nodes, dtype=float)[:, 1:]
        top = np.asarray(top, dtype=np.int64)
        fidx = id2idx[top]
        xz = X[fidx][:, :, [0, 2]]  # [F, 4, 2]
        dt = np.diff(self.time[self.steps:])
        distance = np.zeros(n_t)
        distance[self.steps:] = np.append(0, np.cumsum(load["speed"] * dt))
        d0, d1 = load["direction"]
        if np.isclose(d0, 0):
            ang = 0.5 * np.pi if d1 > 0 else -0.5 * np.pi
        else:
            ang = np.arctan(d1 / d0)
        px = np.cos(ang) * distance + load["start_coord"][0]
        pz = np.sin(ang) * distance + load["start_coord"][1]
        # faces as convex polygons ordered by angle about their mean
        c = xz.mean(axis=1)
        ordv = np.argsort(np.arctan2(xz[:, :, 1] - c[:, None, 1], xz[:, :, 0] - c[:, None, 0]), axis=1)
        poly = np.take_along_axis(xz, ordv[:, :, None], axis=1)
        tree = cKDTree(c)
        k = min(10, len(c))
        _, near = tree.query(np.c_[px, pz], k)
        near = np.atleast_2d(near).reshape(n_t, -1)
        P = poly[near]  # [n_t, k, 4, 2]
        Q = np.roll(P, -1, axis=2)
        cr = (Q[..., 0] - P[..., 0]) * (pz[:, None, None] - P[..., 1]) - (Q[..., 1] - P[..., 1]) * (px[:, None, None] - P[..., 0])
        inside = np.all(cr > 0, axis=2) | np.all(cr < 0, axis=2)
        if not inside.any(axis=1).all():
            raise TypeError("moving_at_plane: the load path leaves the top surface or runs on a face edge")
        act = near[np.arange(n_t), np.argmax(inside, axis=1)]  # first face in nearest order
        cx = xz[act]  # [n_t, 4, 2]
        xd = np.abs(cx[:, :, 0] - px[:, None])
        zd = np.abs(cx[:, :, 1] - pz[:, None])
        with np.errstate(divide="ignore"):
            xw = np.where(np.any(xd < 1e-10, axis=1)[:, None], (xd < 1e-10) * 1.0, 1.0 / xd)
            zw = np.where(np.any(zd < 1e-10, axis=1)[:, None], (zd < 1e-10) * 1.0, 1.0 / zd)
        w = xw * zw
        w = w / w.sum(axis=1, keepdims=True)
        force = np.asarray(self.factor, dtype=float)
        nodal = w[:, :, None] * (force[None, None, :] * sf[:, None, None])  # [n_t, 4, 3]
        dofs = eqmap[fidx[act]]  # [n_t, 4, 3]
        ptr, eqs, vals = [0], [], []
        for t in range(n_t):
            entry = {}
            ok = ~np.isnan(dofs[t])
            for e, v in zip(dofs[t][ok].astype(np.int64), nodal[t][ok]):
                entry[int(e)] = float(v)
            ks = sorted(entry)
            eqs.extend(ks)
            vals.extend(entry[q] for q in ks)
            ptr.append(len(eqs))
        return _table_dropping_zeros(ptr, eqs, vals, self.nb_equations)


def _table_dropping_zeros(ptr, eqs, vals, n_eq):
    ptr = np.asarray(ptr, dtype=np.int64)
    eqs = np.asarray(eqs, dtype=np.int64)
    vals = np.asarray(vals, dtype=float)
    keep = vals != 0.0
    step = np.repeat(np.arange(len(ptr) - 1), np.diff(ptr))
    counts = np.bincount(step[keep], minlength=len(ptr) - 1)
    return ForceTable(np.r_[0, np.cumsum(counts)], eqs[keep], vals[keep], n_eq)


def ricker_table(model, node_id, amplitude, f0, t0, time, direction=1):
    """Point load with a Ricker wavelet, amplitude * (1 - 2 (pi f0 (t - t0))^2) exp(-(pi f0 (t - t0))^2),
    on one node's DOF ``direction`` (a supplied load history; not one of the reference's load
    types, which the solver accepts as a force table)."""
    ids = np.asarray(model.nodes)[:, 0].astype(np.int64)
    idx = int(np.where(ids == int(node_id))[0][0])
    eq = np.asarray(model.eq_nb_dof, dtype=float)[idx, direction]
    if np.isnan(eq):
        raise ValueError("Ricker load on a fixed DOF")
    a = (np.pi * f0 * (np.asarray(time) - t0)) ** 2
    vals = amplitude * (1 - 2 * a) * np.exp(-a)
    n_t = len(time)
    keep = vals != 0
    ptr = np.r_[0, np.cumsum(keep.astype(np.int64))]
    return ForceTable(ptr, np.full(int(keep.sum()), int(eq)), vals[keep], int(model.number_eq))
