// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
//
// The friction-cone program of gorilla-physics' velocity stepping
// (solve_constraint_and_contact, src/dynamics.rs:652-742), which the reference
// hands to Clarabel 0.11.1 (a third-party interior-point solver that is not in
// the repository):
//
//     minimise ½ λᵀ G λ + gᵀ λ   subject to   ‖(λ_t, λ_b)‖ ≤ μ λ_n per contact,
//
// λ = (λ_n, λ_t, λ_b) per contact, μ = 0.95 (Clarabel's A = diag(−μ, −1, −1),
// b = 0, one SecondOrderConeT(3) per contact).  Restated as a primal-dual
// interior-point method with Nesterov–Todd scaling and Mehrotra's
// predictor-corrector (Vandenberghe, "The CVXOPT linear and quadratic cone
// program solvers", 2010, §§ 4-7; Clarabel is of the same family), solved to
// a tighter tolerance than Clarabel's defaults.
#pragma once

namespace orc_socp {

struct Info {
  int iterations = 0;
  double residual = 0.0;  // ‖G λ + g − u‖∞ at exit (u the dual slack)
  double gap = 0.0;       // λᵀu at exit
};

// nc contacts, G row-major (3nc)², returns 0 on convergence, −1 otherwise.
int solve(int nc, const double* G, const double* g, double mu, double* lambda, Info* info);

}  // namespace orc_socp
