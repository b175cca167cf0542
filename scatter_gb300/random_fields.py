"""Random fields on the GPU: per-element log-normal Young's modulus for R realisations.

Drop-in for scatter/random_fields.py ``RF`` on the path the solver needs (the reference
uses gstools' SRF, a third-party package that is not part of this build).  The log-normal
transform and the per-element material update follow random_fields.py:46-118; the field
generator is the seeded randomisation method of csrc/sc_random.cu for the covariance models
the reference offers (random_fields.py:79-88): Gaussian exp(-(pi/4) h^2), Exponential
exp(-h) and Matern (nu = 1, the model's default) of the scaled distance
h = |R^T (x - y) / l|, with l = (aniso_x, 1, aniso_z) * theta as random_fields.py:68 sets it
and R the rotation by ``angles``.  The Linear model is refused in 2D and 3D, where the
triangular covariance is not positive definite (no Gaussian field has it).
"""
import os

import numpy as np
import torch

from . import _native as nat
from . import device as dv


def lognormal_params(mean, sd):
    var = np.log((sd / mean) ** 2 + 1)
    return np.log(mean ** 2 / np.sqrt(mean ** 2 + sd ** 2)), np.sqrt(var)


def element_centroids(model):
    idx = model.node_index()[model.elem]
    return model.nodes[:, 1:][idx].mean(axis=1)


MODEL_CODES = {"Gaussian": 0, "Exponential": 1, "Matern": 2}


def rotation(dim, angles):
    """R (3 x 3) with wave vector k = R kappa for the anisotropy frame rotated by ``angles``:
    Givens rotations in the planes (x, y), (x, z), (y, z) in that order, one angle per plane
    (dim (dim - 1) / 2 of them; a scalar is the first), embedded in 3D."""
    ang = np.zeros(3)
    a = np.atleast_1d(np.asarray(angles, dtype=float))
    n = dim * (dim - 1) // 2
    ang[:min(n, len(a))] = a[:n]
    Rm = np.eye(3)
    for (i, j), th in zip([(0, 1), (0, 2), (1, 2)], ang):
        G = np.eye(3)
        G[i, i] = G[j, j] = np.cos(th)
        G[i, j], G[j, i] = -np.sin(th), np.sin(th)
        Rm = Rm @ G
    return Rm


def lognormal_fields(points, seed, R, lengths, mean, sd, n_modes=1000, model="Gaussian", nu=1.0, angles=0.0,
                     dim=3):
    """Device float32 [n_points, R] (realisation fastest) log-normal values."""
    if model not in MODEL_CODES:
        raise ValueError(f"covariance model {model!r}: the GPU generator draws {sorted(MODEL_CODES)}")
    pts = dv.to_dev(np.asarray(points, dtype=np.float32), torch.float32)
    modes = dv.empty(R * n_modes * 5, torch.float32)
    s = dv.stream_ptr()
    rot = np.ascontiguousarray(rotation(dim, angles), dtype=np.float64)
    nat.call("sc_rf_modes_model", int(seed) & ((1 << 64) - 1), R, n_modes, MODEL_CODES[model], float(nu),
             float(lengths[0]), float(lengths[1]), float(lengths[2]), rot.ctypes.data, modes.data_ptr(), s)
    mu, sig = lognormal_params(mean, sd)
    out = dv.empty(len(points) * R, torch.float32)
    nat.call("sc_rf_lognormal", len(points), pts.data_ptr(), R, n_modes, modes.data_ptr(), float(mu), float(sig),
             out.data_ptr(), s)
    return out.view(len(points), R)


class RF:
    """Same constructor arguments and material-list update as scatter/random_fields.py:8-118."""

    def __init__(self, random_properties, materials, output_folder, element_type):
        self.theta = random_properties["theta"]
        self.seed = random_properties["seed_number"]
        self.materials = materials
        self.material_name = random_properties["material"]
        self.key_material = random_properties["key_material"]
        self.sd = random_properties["std_value"]
        self.aniso_x = random_properties["aniso_x"]
        self.aniso_z = random_properties["aniso_z"]
        self.model_name = random_properties.get("model_name", "Gaussian")
        self.output_folder = output_folder
        self.element_type = element_type
        self.new_material = {}
        self.new_model_material = []
        self.new_material_index = []
        os.makedirs(output_folder, exist_ok=True)

    def generate_gstools_rf(self, nodes, elements, ndim, angles=0.0):
        """Per-element values at the element centroids (random_fields.py:59-118), generated on
        the GPU; the name is the reference's."""
        if self.model_name == "Linear":
            raise ValueError("Linear covariance model: the triangular covariance is valid in 1D only; no Gaussian "
                             f"field in {ndim}D has it")
        if self.model_name not in MODEL_CODES:
            print('model name: "', self.model_name, '" is not supported')  # random_fields.py:87-88
            return None
        seed = abs(self.seed)
        lengths = np.array([self.aniso_x, 1, self.aniso_z]) * self.theta
        mean = self.materials[self.material_name][self.key_material]
        ids = np.asarray(nodes)[:, 0].astype(np.int64)
        id2idx = np.full(int(ids.max()) + 1, -1, dtype=np.int64)
        id2idx[ids] = np.arange(len(ids))
        X = np.asarray(nodes)[:, 1:][id2idx[np.asarray(elements)]].mean(axis=1)
        if ndim == 2:
            X = np.c_[X[:, :2], np.zeros(len(X))]
        self.fields = [dv.host(lognormal_fields(X, seed, 1, lengths, mean, self.sd, model=self.model_name,
                                                angles=angles, dim=ndim))[:, 0].astype(float)]
        for idx in range(len(elements)):
            vals = dict(self.materials[self.material_name])
            vals[self.key_material] = float(self.fields[0][idx])
            self.new_material.update({f"material_{idx + 1}": vals})
            self.new_model_material.append([3, idx, f"material_{idx + 1}"])
            self.new_material_index.append(int(idx))

    generate_rf = generate_gstools_rf

    def update_material_list(self, materials, model, material_idx):
        """random_fields.py:46-57."""
        materials.update(self.new_material)
        for material in model.materials:
            material[1] = material[1] + self.new_material_index[-1]
        model.materials = model.materials + self.new_model_material
        model.materials_index = model.materials_index + self.new_material_index[-1]
        model.materials_index[model.materials_index == material_idx + self.new_material_index[-1]] = \
            self.new_material_index

    def dump(self):
        with open(os.path.join(self.output_folder, "rf_props.txt"), "w") as fo:
            fo.write("Random field properties\n")
            fo.write(f"Model: {self.model_name}\nTheta: {self.theta}\nAniso_x: {self.aniso_x}\n")
            fo.write(f"Aniso_z: {self.aniso_z}\nSeed number: {self.seed}\n")
            fo.write(f"Mean value: {self.materials[self.material_name][self.key_material]}\n")
            fo.write(f"Std value: {self.sd}\nLog normal: True\n")
