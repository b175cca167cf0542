"""GB300-native (sm_103a) finite-element wave-propagation path of PlatypusBytes/scatter.

Drop-in modules mirroring the reference's interface for the hot path:

* ``scatter_gb300.system_matrix.GenerateMatrix`` -- element integration, CSR assembly,
  Lysmer boundaries and Rayleigh damping on the GPU;
* ``scatter_gb300.solvers.NewmarkExplicit`` -- the Newmark time loop (device PCG, CUDA graphs);
* ``scatter_gb300.scatter.scatter`` -- the reference's entry point with the same dictionaries.

The CUDA code is in ``csrc/`` and is exposed through the C ABI of include/scatter_gb300.h.
"""
__all__ = ["build", "system_matrix", "solvers"]
