"""updes_gb300 — GB300-native global RBF collocation (drop-in for Updes' pde_solver).

Public names follow the reference package (updes 1.0.3): clouds, RBFs, nodal
operators, field operators and ``pde_solver`` / ``pde_solver_jit`` returning
``SteadySol(vals, coeffs, mat)``.  Solves run on one GPU through the CUDA
library built by ``updes_gb300/build.py`` (``python -c "import __graft_entry__ as g; g.build()"``).
"""
from .cloud import Cloud, GmshCloud, SquareCloud
from .operators import (
    DEFAULT_OPTIONS, LAST_INFO, CollocationMatrix, SolverOptions, SteadySol, boundary_conditions_func_to_arr,
    capture_operator, compute_coefficients, compute_nb_monomials, core_compute_coefficients, core_gradient_mon,
    core_gradient_rbf, core_laplacian_mon, core_laplacian_rbf, divergence,
    get_field_coefficients, gradient, gradient_vec, laplacian, laplacian_vec, make_all_monomials, make_monomial,
    nodal_div_grad, nodal_gradient, nodal_laplacian, nodal_value, pde_multi_solver, pde_solver, pde_solver_jit,
    pde_solver_many, pde_solver_jit_with_bc, value, value_vec,
)
from .assembly import (assemble_A, assemble_B, assemble_bd_Phi_P, assemble_invert_A, assemble_op_Phi_P, assemble_P,
                       assemble_Phi, assemble_q, gaussian_func, inv_multiquadric_func, make_nodal_rbf,
                       multiquadric_func, polyharmonic_func, thin_plate_func)
from .batched import PanelTuner, pde_solver_batched
from .fields import (apply_neumann_conditions, cartesian_gradient, cartesian_gradient_vec, divergence_vec, dot_mat,
                     dot_vec, duplicate_robin_coeffs, enforce_cartesian_gradient_neumann, gradient_vals,
                     gradient_vals_vec, integrate_field, interpolate_field, laplacian_vals, laplacian_vals_vec,
                     zerofy_periodic_cond)
from .rbf import distance, gaussian, inverse_multiquadric, multiquadric, polyharmonic, rbf_spec, thin_plate

# the reference's names of its un-jitted vmaps (updes/operators.py:149, 186, 207, 370)
value_vec_, gradient_vec_, gradient_vals_vec_, laplacian_vals_vec_ = (value_vec, gradient_vec, gradient_vals_vec,
                                                                      laplacian_vals_vec)

__version__ = "0.1.0"
