"""CPU oracle for the scatter finite-element wave-propagation path.

TEST INFRASTRUCTURE ONLY.  This package is a plain numpy/scipy (and C, for the
timed CPU baseline) restatement of the reference algorithm, used as the checker
for the CUDA path.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.  The
product package ``scatter_gb300`` never imports, links or executes anything in
here.

Every function cites the reference file:line it restates.  The restatement is
pinned against the reference's own golden vectors (``tests/golden``): element
matrices, assembled K/M/C, absorbing-boundary matrices and force tables produced
by the reference's own code, and the reference's shipped time histories
(integration_tests/test_data/*.pickle, results_mean_2d, results_mean/VTK).

Modules
-------
elements   shape functions, Gauss rules, D matrix, element Ke/Me, face matrices
assembly   element-order COO -> CSR assembly and the reference's zero semantics
lysmer     absorbing boundaries with the reference's node-order behaviour
loads      pulse / heaviside / moving / moving_at_plane force tables
newmark    average-acceleration Newmark (beta=1/4, gamma=1/2) with a direct solve
explicit   central-difference, row-sum lumped mass (the explicit scheme's oracle)
mesh       gmsh 2.2 reader, boundary planes, equation numbering
"""
