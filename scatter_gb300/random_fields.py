"""Random fields on the GPU: per-element log-normal Young's modulus for R realisations.

Drop-in for scatter/random_fields.py ``RF`` on the path the solver needs (the reference
uses gstools' SRF, a third-party package that is not part of this build).  The log-normal
transform and the per-element material update follow random_fields.py:46-118; the field
generator is the seeded randomisation method of csrc/sc_random.cu (Gaussian covariance
exp(-(pi/4)|r/l|^2) with l = (aniso_x, 1, aniso_z) * theta as random_fields.py:68 sets it).
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


def lognormal_fields(points, seed, R, lengths, mean, sd, n_modes=1000):
    """Device float32 [n_points, R] (realisation fastest) log-normal values."""
    pts = dv.to_dev(np.asarray(points, dtype=np.float32), torch.float32)
    modes = dv.empty(R * n_modes * 5, torch.float32)
    s = dv.stream_ptr()
    nat.call("sc_rf_modes", int(seed) & ((1 << 64) - 1), R, n_modes, float(lengths[0]), float(lengths[1]),
             float(lengths[2]), modes.data_ptr(), s)
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
        if self.model_name != "Gaussian":
            raise NotImplementedError("only the Gaussian covariance model is generated on the GPU")
        os.makedirs(output_folder, exist_ok=True)

    def generate_rf(self, nodes, elements, ndim, model=None):
        seed = abs(self.seed)
        lengths = np.array([self.aniso_x, 1, self.aniso_z]) * self.theta
        mean = self.materials[self.material_name][self.key_material]
        ids = np.asarray(nodes)[:, 0].astype(np.int64)
        id2idx = np.full(int(ids.max()) + 1, -1, dtype=np.int64)
        id2idx[ids] = np.arange(len(ids))
        X = np.asarray(nodes)[:, 1:][id2idx[np.asarray(elements)]].mean(axis=1)
        if ndim == 2:
            X = np.c_[X[:, :2], np.zeros(len(X))]
        self.fields = [dv.host(lognormal_fields(X, seed, 1, lengths, mean, self.sd))[:, 0].astype(float)]
        for idx in range(len(elements)):
            vals = dict(self.materials[self.material_name])
            vals[self.key_material] = float(self.fields[0][idx])
            self.new_material.update({f"material_{idx + 1}": vals})
            self.new_model_material.append([3, idx, f"material_{idx + 1}"])
            self.new_material_index.append(int(idx))

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
