"""Force tables restated (oracle; test infrastructure only).

Restates Force.initialise_load / update_load_at_t (scatter/force_external.py:19-349)
as a dense table ``F[n_t, n_eq]`` (small cases) or a sparse (step, eq, value)
list.  ``ini_steps`` defaults to 5 (scatter/validator.py:57).
"""
import numpy as np


def time_grid(T, dt):
    """scatter/scatter.py:117."""
    return np.linspace(0, T, int(np.ceil(T / dt) + 1))


def step_factors(kind, n_t, steps):
    """force_external.py:76-96 (pulse, heaviside), :113-115 and :158-160 (moving ramps)."""
    if n_t <= steps:
        raise SystemExit("Error: Number of loading steps smaller than " + str(steps))
    if kind == "pulse":
        return np.append(np.linspace(0, 1, int((steps - 1) / 2), endpoint=False),
                         np.linspace(1, 0, int((steps + 1) / 2)))
    f = np.ones(n_t)
    f[:steps] = np.linspace(0, 1, steps)
    return f


def _node_eqs(model, node_id):
    ids = np.asarray(model["nodes"])[:, 0].astype(int)
    idx = int(np.where(ids == int(node_id))[0][0])
    return np.asarray(model["eq_nb_dof"], dtype=float)[idx]


def table(load, time, model, top_surface=None):
    """Dense force table [n_t, n_eq] for pulse / heaviside / moving / moving_at_plane."""
    n_eq = int(model["number_eq"])
    n_t = len(time)
    steps = load.get("ini_steps", 5)
    kind = load["type"]
    factor = load.get("force")
    F = np.zeros((n_t, n_eq))
    if kind in ("pulse", "heaviside"):  # force_external.py:250-279
        sf = step_factors(kind, n_t, steps)
        for t in range(n_t):
            if kind == "pulse" and not t < steps - 1:
                continue
            for n in load["node"]:
                for i, eq in enumerate(_node_eqs(model, n)):
                    if not np.isnan(eq):
                        F[t, int(eq)] = float(factor[i]) * sf[t]
        return F
    if kind == "moving":  # force_external.py:98-149, :320-345
        sf = step_factors(kind, n_t, steps)
        nodes = np.asarray(model["nodes"], dtype=float)
        idx = int(np.where(nodes[:, 0] == load["node"])[0][0])
        lst = np.where((nodes[:, 1] == nodes[idx, 1]) & (nodes[:, 2] == nodes[idx, 2]))[0]
        dist = np.sqrt((nodes[lst, 3] - nodes[idx, 3]) ** 2)
        lst = lst[np.argsort(dist)]
        dist = np.sort(dist)
        speed = np.ones(n_t) * load["speed"]
        speed[:steps] = 0
        ld = speed * (time - time[steps])
        eqmap = np.asarray(model["eq_nb_dof"], dtype=float)
        for t in range(n_t):
            if ld[t] >= np.max(dist):
                continue
            idn = np.where(dist <= ld[t])[0][-1]
            x = ld[t] - nodes[lst[idn], 3] + nodes[lst[0], 3]
            length = dist[idn + 1] - dist[idn]
            shp = np.array([1 - x / length, x * length])  # as written at force_external.py:337-338
            for j, ni in enumerate((lst[idn], lst[idn + 1])):
                for i, eq in enumerate(eqmap[ni]):
                    if not np.isnan(eq):
                        F[t, int(eq)] = float(factor[i]) * shp[j] * sf[t]
        return F
    if kind == "moving_at_plane":  # force_external.py:151-211, :281-318
        sf = step_factors(kind, n_t, steps)
        nodes = np.asarray(model["nodes"], dtype=float)
        eqmap = np.asarray(model["eq_nb_dof"], dtype=float)
        top = np.asarray(top_surface, dtype=np.int64)
        xz = nodes[top - 1][:, :, [1, 3]]
        dt = np.diff(time[steps:])
        distance = np.zeros(n_t)
        distance[steps:] = np.append(0, np.cumsum(load["speed"] * dt))
        d0, d1 = load["direction"]
        if np.isclose(d0, 0):
            ang = 0.5 * np.pi if d1 > 0 else -0.5 * np.pi
        else:
            ang = np.arctan(d1 / d0)
        px = np.cos(ang) * distance + load["start_coord"][0]
        pz = np.sin(ang) * distance + load["start_coord"][1]
        for t in range(n_t):
            act = _find_face(xz, px[t], pz[t])
            if act is None:
                raise TypeError("moving_at_plane: load outside the top surface")
            c = xz[act]
            xd = np.abs(c[:, 0] - px[t])
            zd = np.abs(c[:, 1] - pz[t])
            xw = (xd < 1e-10) * 1 if np.any(xd < 1e-10) else 1 / xd
            zw = (zd < 1e-10) * 1 if np.any(zd < 1e-10) else 1 / zd
            w = xw * zw
            w = w / w.sum()
            nf = w[:, None] * (np.asarray(factor, dtype=float) * sf[t])[None, :]
            dofs = eqmap[top[act] - 1]
            ok = ~np.isnan(dofs)
            F[t, dofs[ok].astype(int)] = nf[ok]
        return F
    raise SystemExit(f"Error: Load type {kind} not supported")


def _find_face(xz, x, z):
    """First top face (in the reference's KD-tree nearest-centroid order, which for
    convex, non-overlapping faces is the unique face) strictly containing (x, z)."""
    c = xz.mean(axis=1)
    order = np.argsort((c[:, 0] - x) ** 2 + (c[:, 1] - z) ** 2, kind="stable")[:10]
    for f in order:
        p = xz[f]
        m = p.mean(axis=0)
        p = p[np.argsort(np.arctan2(p[:, 1] - m[1], p[:, 0] - m[0]))]
        q = np.roll(p, -1, axis=0)
        cr = (q[:, 0] - p[:, 0]) * (z - p[:, 1]) - (q[:, 1] - p[:, 1]) * (x - p[:, 0])
        if np.all(cr > 0) or np.all(cr < 0):
            return int(f)
    return None
