// oracle.cpp -- FP64 CPU restatement of ssim's FEM time-stepping path.
//
// TEST INFRASTRUCTURE ONLY: this file is the checker for the CUDA library and
// the timed CPU baseline.  The product library never links or calls it.
//
// Citations are to files of the ssim reference project (paths within that
// project).  The numeric core of the reference (`mathprim`: COO->CSR, gather
// operator, CG, Newton, L-BFGS, line search) is an un-vendored, unpinned
// dependency; where this file restates one of its algorithms it says so and
// states the definition used (those trajectories are "parity unpinned").
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using Vec = std::vector<double>;

// ---------------------------------------------------------------------------
// small dense helpers (row-major 3x3)
// ---------------------------------------------------------------------------
inline double det3(const double* A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}

// inverse via the adjugate (Eigen's fixed 3x3 inverse is also cofactor based)
inline void inv3(const double* A, double* B) {
  const double d = det3(A);
  const double id = 1.0 / d;
  B[0] = (A[4] * A[8] - A[5] * A[7]) * id;
  B[1] = (A[2] * A[7] - A[1] * A[8]) * id;
  B[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  B[3] = (A[5] * A[6] - A[3] * A[8]) * id;
  B[4] = (A[0] * A[8] - A[2] * A[6]) * id;
  B[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  B[6] = (A[3] * A[7] - A[4] * A[6]) * id;
  B[7] = (A[1] * A[6] - A[0] * A[7]) * id;
  B[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

inline void cross(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// cofactor matrix = dJ/dF.  ssim's partial_determinant (internal_physic.hpp:41-48) takes the
// columns of its argument; the model receives F transposed (def_grad = cmap(F view)), so in
// terms of the row-major F the rows of cof(F) are cross products of the rows of F.
inline void cofactor(const double* F, double* C) {
  cross(F + 3, F + 6, C + 0);
  cross(F + 6, F + 0, C + 3);
  cross(F + 0, F + 3, C + 6);
}

// ---------------------------------------------------------------------------
// stable Neo-Hookean (stable_neohookean.hpp:23-111, basic_elast.hpp:10-20)
// ---------------------------------------------------------------------------
constexpr double kDelta = 1.0;  // delta(lambda, mu) == 1 in 3D (stable_neohookean.hpp:93-104)

inline double snh_alpha(double lambda, double mu) { return (1.0 - 1.0 / (3.0 + kDelta)) * mu / lambda + 1.0; }

inline double snh_energy(const double* F, double lambda, double mu) {
  double Ic = 0;
  for (int i = 0; i < 9; ++i) Ic += F[i] * F[i];
  const double alpha = snh_alpha(lambda, mu);
  const double Jm = det3(F) - alpha;
  const double zero_energy = 0.5 * (lambda * (1 - alpha) * (1 - alpha) - mu * std::log(3.0 + kDelta));
  return 0.5 * (mu * (Ic - 3.0) + lambda * Jm * Jm - mu * std::log(Ic + kDelta)) - zero_energy;
}

inline double snh_stress(const double* F, double lambda, double mu, double* P) {
  double Ic = 0;
  for (int i = 0; i < 9; ++i) Ic += F[i] * F[i];
  const double alpha = snh_alpha(lambda, mu);
  const double Jm = det3(F) - alpha;
  double C[9];
  cofactor(F, C);
  const double s = mu * (1.0 - 1.0 / (Ic + kDelta));
  for (int i = 0; i < 9; ++i) P[i] = lambda * Jm * C[i] + s * F[i];
  const double zero_energy = 0.5 * (lambda * (1 - alpha) * (1 - alpha) - mu * std::log(3.0 + kDelta));
  return 0.5 * (mu * (Ic - 3.0) + lambda * Jm * Jm - mu * std::log(Ic + kDelta)) - zero_energy;
}

// sum of the magnitudes of the terms of snh_energy: the scale of its absolute round-off (the terms are
// O(mu) and cancel to O(mu strain^2), so the round-off of Psi is relative to this, not to Psi)
inline double snh_energy_scale(const double* F, double lambda, double mu) {
  double Ic = 0;
  for (int i = 0; i < 9; ++i) Ic += F[i] * F[i];
  const double alpha = snh_alpha(lambda, mu);
  const double Jm = det3(F) - alpha;
  const double zero_energy = 0.5 * (lambda * (1 - alpha) * (1 - alpha) - mu * std::log(3.0 + kDelta));
  return 0.5 * (mu * std::fabs(Ic - 3.0) + lambda * Jm * Jm + mu * std::fabs(std::log(Ic + kDelta))) +
         std::fabs(zero_energy);
}

// x_hat (internal_physic.hpp:59-63): the cross-product matrix [v]x.
inline void xhat(const double* v, double s, double* M) {
  M[0] = 0;
  M[1] = -v[2] * s;
  M[2] = v[1] * s;
  M[3] = v[2] * s;
  M[4] = 0;
  M[5] = -v[0] * s;
  M[6] = -v[1] * s;
  M[7] = v[0] * s;
  M[8] = 0;
}

// 9x9 Hessian, index i = r*3 + c of the row-major F (stable_neohookean.hpp:64-91 with add_HJ
// internal_physic.hpp:66-76 applied to the transposed argument, see cofactor()).
inline void snh_hessian(const double* F, double lambda, double mu, double* H) {
  double I2 = 0;
  for (int i = 0; i < 9; ++i) I2 += F[i] * F[i];
  const double I3 = det3(F);
  const double alpha = snh_alpha(lambda, mu);
  const double scale = lambda * (I3 - alpha);
  double g[9];
  cofactor(F, g);
  const double a = mu * (1.0 - 1.0 / (I2 + kDelta));
  const double b = mu * (2.0 / (I2 + kDelta) / (I2 + kDelta));
  for (int i = 0; i < 9; ++i)
    for (int j = 0; j < 9; ++j) H[i * 9 + j] = (i == j ? a : 0.0) + b * F[i] * F[j] + lambda * g[i] * g[j];
  // add_HJ on blocks indexed by rows of F
  double f0[9], f1[9], f2[9];
  xhat(F + 0, scale, f0);
  xhat(F + 3, scale, f1);
  xhat(F + 6, scale, f2);
  auto add_block = [&](int R, int Cc, const double* M, double sgn) {
    for (int m = 0; m < 3; ++m)
      for (int n = 0; n < 3; ++n) H[(3 * R + m) * 9 + 3 * Cc + n] += sgn * M[m * 3 + n];
  };
  add_block(1, 0, f2, +1);
  add_block(0, 1, f2, -1);
  add_block(2, 0, f1, -1);
  add_block(0, 2, f1, +1);
  add_block(2, 1, f0, +1);
  add_block(1, 2, f0, -1);
}

// ---------------------------------------------------------------------------
// cyclic Jacobi eigensolver (Golub & Van Loan, "Matrix Computations", Alg. 8.5.3 with the
// symmetric 2x2 Schur rotation 8.5.1).  Replaces Eigen::SelfAdjointEigenSolver used at
// time_step.hpp:51; the projection V*max(L,eps)*V^T is a spectral function, so any
// accurate eigensolver gives the same result to round-off.
// ---------------------------------------------------------------------------
int sym_eigen(int n, const double* Ain, double* w, double* V) {
  double A[144];
  std::memcpy(A, Ain, sizeof(double) * n * n);
  for (int i = 0; i < n * n; ++i) V[i] = 0;
  for (int i = 0; i < n; ++i) V[i * n + i] = 1;
  double fro = 0;
  for (int i = 0; i < n * n; ++i) fro += A[i] * A[i];
  fro = std::sqrt(fro);
  int sweep = 0;
  for (; sweep < 100; ++sweep) {
    double off = 0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += 2 * A[p * n + q] * A[p * n + q];
    if (std::sqrt(off) <= 1e-16 * fro || off == 0.0) break;
    for (int p = 0; p < n; ++p) {
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p * n + q];
        if (apq == 0.0) continue;
        const double tau = (A[q * n + q] - A[p * n + p]) / (2 * apq);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1 + tau * tau));
        const double c = 1 / std::sqrt(1 + t * t), s = t * c;
        for (int k = 0; k < n; ++k) {  // A <- A J (columns p, q)
          const double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // A <- J^T A (rows p, q)
          const double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {  // V <- V J
          const double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
    }
  }
  for (int i = 0; i < n; ++i) w[i] = A[i * n + i];
  return sweep;
}

// wrapped_pfpx make_spsd branch (time_step.hpp:50-56): eigenvalues clamped to >= eps (absolute).
void project_spd(const double* H, double eps, double* Hp) {
  double w[9], V[81];
  sym_eigen(9, H, w, V);
  for (int i = 0; i < 9; ++i) w[i] = std::max(w[i], eps);
  for (int i = 0; i < 9; ++i)
    for (int j = 0; j < 9; ++j) {
      double s = 0;
      for (int k = 0; k < 9; ++k) s += V[i * 9 + k] * w[k] * V[j * 9 + k];
      Hp[i * 9 + j] = s;
    }
}

// D(v, j) = dF(a, j)/dx_{v,a}: the constant dF/dx of compute_pfpx_3 (internal_physic.hpp:107-160)
// with Dminv(r, c) the row-major inverse of Dm.
inline void shape_grads(const double* Dm, double D[4][3]) {
  for (int j = 0; j < 3; ++j) {
    D[1][j] = Dm[0 * 3 + j];
    D[2][j] = Dm[1 * 3 + j];
    D[3][j] = Dm[2 * 3 + j];
    D[0][j] = -(Dm[0 * 3 + j] + Dm[1 * 3 + j] + Dm[2 * 3 + j]);
  }
}

// ---------------------------------------------------------------- linear elasticity
// elast::linear (linear.hpp:23-68): eps = (F + F^T)/2 - I (approx_green_strain, internal_physic.hpp:27-30),
// Psi = mu |eps|^2 + lambda/2 tr(eps)^2, P = 2 mu eps + lambda tr(eps) I,
// H = mu I + mu [(i,j),(j,i)] + lambda [(i,i),(j,j)] (row-major flat index i*3+j).
inline double linear_energy(const double* F, double lambda, double mu) {
  double n2 = 0, tr = 0;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      const double e = 0.5 * (F[r * 3 + c] + F[c * 3 + r]) - (r == c ? 1.0 : 0.0);
      n2 += e * e;
      if (r == c) tr += e;
    }
  return mu * n2 + 0.5 * lambda * tr * tr;
}

inline double linear_stress(const double* F, double lambda, double mu, double* P) {
  double eps[9], tr = 0;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      eps[r * 3 + c] = 0.5 * (F[r * 3 + c] + F[c * 3 + r]) - (r == c ? 1.0 : 0.0);
      if (r == c) tr += eps[r * 3 + c];
    }
  for (int k = 0; k < 9; ++k) P[k] = 2 * mu * eps[k] + (k % 4 == 0 ? lambda * tr : 0.0);
  return linear_energy(F, lambda, mu);
}

inline void linear_hessian(double lambda, double mu, double* H) {
  for (int k = 0; k < 81; ++k) H[k] = 0;
  for (int k = 0; k < 9; ++k) H[k * 9 + k] = mu;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      H[(i * 3 + j) * 9 + (j * 3 + i)] += mu;
      H[(i * 3 + i) * 9 + (j * 3 + j)] += lambda;
    }
}

// the elastic model of a time step: 0 stable Neo-Hookean, 1 linear
inline double model_energy(int model, const double* F, double l, double m) {
  return model == 1 ? linear_energy(F, l, m) : snh_energy(F, l, m);
}
inline double model_stress(int model, const double* F, double l, double m, double* P) {
  return model == 1 ? linear_stress(F, l, m, P) : snh_stress(F, l, m, P);
}
// the scale of the energy's round-off (the linear energy's terms are all non-negative)
inline double model_energy_scale(int model, const double* F, double l, double m) {
  return model == 1 ? linear_energy(F, l, m) : snh_energy_scale(F, l, m);
}
inline void model_hessian(int model, const double* F, double l, double m, double* H) {
  if (model == 1)
    linear_hessian(l, m, H);
  else
    snh_hessian(F, l, m, H);
}

// K = pfpx^T * H * pfpx (time_step.hpp:58); rows/cols vertex*3 + dof.
void element_stiffness(const double* F, const double* Dminv, double lambda, double mu, bool make_spsd,
                       double* K, int model = 0) {
  double H[81], Hp[81];
  model_hessian(model, F, lambda, mu, H);
  const double* Hu = H;
  if (make_spsd) {
    project_spd(H, 1e-3, Hp);
    Hu = Hp;
  }
  double D[4][3];
  shape_grads(Dminv, D);
  for (int v = 0; v < 4; ++v)
    for (int a = 0; a < 3; ++a)
      for (int w = 0; w < 4; ++w)
        for (int b = 0; b < 3; ++b) {
          double s = 0;
          for (int j = 0; j < 3; ++j)
            for (int l = 0; l < 3; ++l) s += D[v][j] * Hu[(a * 3 + j) * 9 + b * 3 + l] * D[w][l];
          K[(v * 3 + a) * 12 + w * 3 + b] = s;
        }
}

// ---------------------------------------------------------------- 2D (triangles in the plane)
// stable_neohookean<2> (stable_neohookean.hpp:23-104): delta = the positive root of
// (2t+1) d^2 + (2t+2) d - 2t = 0, t = mu/lambda; alpha = (1 - 1/(2 + delta)) mu/lambda + 1;
// Psi = (mu (Ic - 2) + lambda (J - alpha)^2 - mu log(Ic + delta))/2 - (lambda (1-alpha)^2 - mu log(2 + delta))/2;
// P = lambda (J - alpha) dJ/dF + mu (1 - 1/(Ic + delta)) F with dJ/dF = [[F11, -F10], [-F01, F00]];
// H = mu (1 - 1/(Ic+delta)) I + 2 mu/(Ic+delta)^2 f f^T + lambda g g^T + lambda (J - alpha) d2J/dF2
// (internal_physic.hpp:33-54 partial_determinant / add_HJ); F row-major, flat index r*2+c.
inline double snh2_delta(double lambda, double mu) {
  const double t = mu / lambda, a = 2 * t + 1, b = 2 * t + 2, c = -2 * t;
  return (-b + std::sqrt(b * b - 4 * a * c)) / (2 * a);
}
inline double snh2_alpha(double lambda, double mu) {
  return (1 - 1 / (2 + snh2_delta(lambda, mu))) * mu / lambda + 1;
}
inline double snh2_energy(const double* F, double lambda, double mu) {
  const double del = snh2_delta(lambda, mu), alpha = snh2_alpha(lambda, mu);
  const double Ic = F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3];
  const double Jm = F[0] * F[3] - F[1] * F[2] - alpha;
  const double zero = 0.5 * (lambda * (1 - alpha) * (1 - alpha) - mu * std::log(2 + del));
  return 0.5 * (mu * (Ic - 2) + lambda * Jm * Jm - mu * std::log(Ic + del)) - zero;
}
inline double snh2_energy_scale(const double* F, double lambda, double mu) {
  const double del = snh2_delta(lambda, mu), alpha = snh2_alpha(lambda, mu);
  const double Ic = F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3];
  const double Jm = F[0] * F[3] - F[1] * F[2] - alpha;
  const double zero = 0.5 * (lambda * (1 - alpha) * (1 - alpha) - mu * std::log(2 + del));
  return 0.5 * (mu * std::fabs(Ic - 2) + lambda * Jm * Jm + mu * std::fabs(std::log(Ic + del))) + std::fabs(zero);
}
inline double snh2_stress(const double* F, double lambda, double mu, double* P) {
  const double del = snh2_delta(lambda, mu), alpha = snh2_alpha(lambda, mu);
  const double Ic = F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3];
  const double Jm = F[0] * F[3] - F[1] * F[2] - alpha;
  const double dJ[4] = {F[3], -F[2], -F[1], F[0]};
  const double c = mu * (1.0 - 1.0 / (Ic + del));
  for (int k = 0; k < 4; ++k) P[k] = lambda * Jm * dJ[k] + c * F[k];
  return snh2_energy(F, lambda, mu);
}
inline void snh2_hessian(const double* F, double lambda, double mu, double* H) {
  const double del = snh2_delta(lambda, mu), alpha = snh2_alpha(lambda, mu);
  const double Ic = F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3];
  const double J = F[0] * F[3] - F[1] * F[2];
  const double g[4] = {F[3], -F[2], -F[1], F[0]};
  const double a = mu * (1.0 - 1.0 / (Ic + del)), b = mu * 2.0 / ((Ic + del) * (Ic + del));
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) H[i * 4 + j] = (i == j ? a : 0.0) + b * F[i] * F[j] + lambda * g[i] * g[j];
  const double sc = lambda * (J - alpha);
  H[0 * 4 + 3] += sc;
  H[3 * 4 + 0] += sc;
  H[1 * 4 + 2] -= sc;
  H[2 * 4 + 1] -= sc;
}
// elast::linear<2> (linear.hpp:23-68) with the 2x2 approx_green_strain
inline double linear2_energy(const double* F, double lambda, double mu) {
  const double e00 = F[0] - 1, e11 = F[3] - 1, e01 = 0.5 * (F[1] + F[2]);
  const double tr = e00 + e11;
  return mu * (e00 * e00 + e11 * e11 + 2 * e01 * e01) + 0.5 * lambda * tr * tr;
}
inline double linear2_stress(const double* F, double lambda, double mu, double* P) {
  const double e00 = F[0] - 1, e11 = F[3] - 1, e01 = 0.5 * (F[1] + F[2]);
  const double tr = e00 + e11;
  P[0] = 2 * mu * e00 + lambda * tr;
  P[1] = 2 * mu * e01;
  P[2] = 2 * mu * e01;
  P[3] = 2 * mu * e11 + lambda * tr;
  return linear2_energy(F, lambda, mu);
}
inline void linear2_hessian(double lambda, double mu, double* H) {
  for (int k = 0; k < 16; ++k) H[k] = 0;
  for (int k = 0; k < 4; ++k) H[k * 4 + k] = mu;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      H[(i * 2 + j) * 4 + (j * 2 + i)] += mu;
      H[(i * 2 + i) * 4 + (j * 2 + j)] += lambda;
    }
}
inline double model2_energy(int model, const double* F, double l, double m) {
  return model == 1 ? linear2_energy(F, l, m) : snh2_energy(F, l, m);
}
inline double model2_stress(int model, const double* F, double l, double m, double* P) {
  return model == 1 ? linear2_stress(F, l, m, P) : snh2_stress(F, l, m, P);
}
inline double model2_energy_scale(int model, const double* F, double l, double m) {
  return model == 1 ? linear2_energy(F, l, m) : snh2_energy_scale(F, l, m);
}
inline void model2_hessian(int model, const double* F, double l, double m, double* H) {
  if (model == 1)
    linear2_hessian(l, m, H);
  else
    snh2_hessian(F, l, m, H);
}
// the 6x6 triangle stiffness pfpx^T H pfpx (compute_pfpx_2, internal_physic.hpp:79-104), embedded in 3 dofs
// per vertex (z rows and columns zero): K[(v*3+a)*9 + w*3+b]
void element_stiffness_2d(const double* F, const double* Dm, double lambda, double mu, bool make_spsd, double* K,
                          int model) {
  double H[16], w[4], V[16];
  model2_hessian(model, F, lambda, mu, H);
  if (make_spsd) {
    sym_eigen(4, H, w, V);
    for (int i = 0; i < 4; ++i) w[i] = std::max(w[i], 1e-3);
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        double t = 0;
        for (int k = 0; k < 4; ++k) t += V[i * 4 + k] * w[k] * V[j * 4 + k];
        H[i * 4 + j] = t;
      }
  }
  double D[3][2];
  for (int j = 0; j < 2; ++j) {
    D[1][j] = Dm[0 * 2 + j];
    D[2][j] = Dm[1 * 2 + j];
    D[0][j] = -(Dm[0 * 2 + j] + Dm[1 * 2 + j]);
  }
  for (int k = 0; k < 81; ++k) K[k] = 0;
  for (int v = 0; v < 3; ++v)
    for (int a = 0; a < 2; ++a)
      for (int wv = 0; wv < 3; ++wv)
        for (int b = 0; b < 2; ++b) {
          double t = 0;
          for (int j = 0; j < 2; ++j)
            for (int l = 0; l < 2; ++l) t += D[v][j] * H[(a * 2 + j) * 4 + b * 2 + l] * D[wv][l];
          K[(v * 3 + a) * 9 + wv * 3 + b] = t;
        }
}
// p1_element_2d (bilinears.hpp:45-96): |det J| = 2 area; mass |det J| {1/12, 1/24} rho; Laplacian
// alpha area grad phi_i . grad phi_j
void element_mass_2d(const double* Xv[3], double rho, double M[9]) {
  const double J[4] = {Xv[1][0] - Xv[0][0], Xv[2][0] - Xv[0][0], Xv[1][1] - Xv[0][1], Xv[2][1] - Xv[0][1]};
  const double detJ = std::fabs(J[0] * J[3] - J[1] * J[2]);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M[i * 3 + j] = (detJ * (i == j ? 1.0 / 12 : 1.0 / 24)) * rho;
}
void element_laplace_2d(const double* Xv[3], double alpha, double L[9]) {
  const double J[4] = {Xv[1][0] - Xv[0][0], Xv[2][0] - Xv[0][0], Xv[1][1] - Xv[0][1], Xv[2][1] - Xv[0][1]};
  const double det = J[0] * J[3] - J[1] * J[2];
  const double iJ[4] = {J[3] / det, -J[1] / det, -J[2] / det, J[0] / det};
  double g[3][2];
  for (int k = 0; k < 2; ++k) {
    g[1][k] = iJ[0 * 2 + k];
    g[2][k] = iJ[1 * 2 + k];
    g[0][k] = -(g[1][k] + g[2][k]);
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) L[i * 3 + j] = alpha * std::fabs(det) / 2.0 * (g[i][0] * g[j][0] + g[i][1] * g[j][1]);
}

// ---------------------------------------------------------------------------
// BLAS-1 helpers
// ---------------------------------------------------------------------------
double dot(const Vec& a, const Vec& b) {
  double s = 0;
  const long n = (long)a.size();
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (long i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}
double nrm2(const Vec& a) { return std::sqrt(dot(a, a)); }

}  // namespace

// ===========================================================================
// time-step object: basic_time_step (time_step.hpp:168-715)
// ===========================================================================
struct orc_ts {
  int nv = 0, nt = 0, n = 0;
  Vec X;                     // [nv*3] rest positions
  std::vector<int32_t> cells;  // [nt*4]
  double dt, E, nu, rho, damping = 0.0, rtol = 1e-2, abs_tol = 1e-2, mass_third = 0.0;
  Vec E_elem, nu_elem;       // optional per-element material
  int pd_diff_mode = 0;
  std::vector<int8_t> dof_type;  // [nv*3]
  Vec dbc_values, deformation, prev_deform, inertia, next, velocity, ext_accel, forces;
  Vec dminv, vol, defgrad, local_energy, local_force, local_K;
  // CSR (identical pattern for mass, system and PD matrices)
  std::vector<int32_t> row_ptr, col_idx;
  Vec ncg_L;                  // NCG preconditioner factor on the CSR pattern (empty: identity)
  int model = 0;              // elastic model: 0 stable Neo-Hookean, 1 linear
  int cv = 4;                 // vertices per cell: 4 (tets), 3 (triangles in the plane) or 2 (springs)
  bool springs = false;       // mass-spring system: cells are springs, lumped vertex masses
  bool tri2d = false;         // 2D triangles: x, y dofs (the z dof of every vertex carries no force)
  Vec sp_rest, sp_k, vmass;
  Vec mass_vals, massf_vals, sys_vals, pd_vals;
  std::vector<int32_t> hess_dst;            // [nt*144] CSR slot of each local entry
  std::vector<int32_t> hcon_ptr, hcon_src;  // per CSR slot, the local entries that add into it
  std::vector<int32_t> fcon_ptr, fcon_src;  // per vertex, the (elem*4+i) that add into it
  bool has_reset = false;
  bool pd_ready = false;
  double energy_scale = 0;  // sum of term magnitudes of the last energy evaluation (line-search slack)

  double lam(int e) const {
    const double Ee = E_elem.empty() ? E : E_elem[e];
    const double ne = nu_elem.empty() ? nu : nu_elem[e];
    return Ee * ne / ((1 + ne) * (1 - 2 * ne));
  }
  double mu(int e) const {
    const double Ee = E_elem.empty() ? E : E_elem[e];
    const double ne = nu_elem.empty() ? nu : nu_elem[e];
    return Ee / (2 * (1 + ne));
  }
  bool dbc(int dof) const { return dof_type[dof] == 1; }
};

namespace {

// CSR pattern of local_global_composer::hessian (global_composer.hpp:68-100): the union over tets
// of (3*cell[i]+a, 3*cell[j]+b), rows ascending, columns strictly ascending, full storage.  The
// enumeration order of the CSR is the offset map of global_composer.hpp:94-100.
void build_pattern(orc_ts& s) {
  const int cv = s.cv, L = 3 * cv, LL = L * L;
  std::vector<std::vector<int32_t>> nb(s.nv);
  for (int e = 0; e < s.nt; ++e)
    for (int i = 0; i < cv; ++i)
      for (int j = 0; j < cv; ++j) nb[s.cells[e * cv + i]].push_back(s.cells[e * cv + j]);
  for (auto& v : nb) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
  }
  s.row_ptr.assign(s.n + 1, 0);
  for (int u = 0; u < s.nv; ++u)
    for (int a = 0; a < 3; ++a) s.row_ptr[3 * u + a + 1] = 3 * (int)nb[u].size();
  for (int r = 0; r < s.n; ++r) s.row_ptr[r + 1] += s.row_ptr[r];
  s.col_idx.resize(s.row_ptr[s.n]);
  for (int u = 0; u < s.nv; ++u)
    for (int a = 0; a < 3; ++a) {
      int o = s.row_ptr[3 * u + a];
      for (int w : nb[u])
        for (int b = 0; b < 3; ++b) s.col_idx[o++] = 3 * w + b;
    }
  // element-local -> CSR slot map (global_composer.hpp:103-119)
  s.hess_dst.resize((size_t)s.nt * LL);
  for (int e = 0; e < s.nt; ++e)
    for (int i = 0; i < cv; ++i) {
      const int u = s.cells[e * cv + i];
      for (int j = 0; j < cv; ++j) {
        const int w = s.cells[e * cv + j];
        const int k = (int)(std::lower_bound(nb[u].begin(), nb[u].end(), w) - nb[u].begin());
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b)
            s.hess_dst[(size_t)e * LL + (i * 3 + a) * L + j * 3 + b] = s.row_ptr[3 * u + a] + 3 * k + b;
      }
    }
  // invert: per slot, its contributing local entries (in element order)
  const int nnz = s.row_ptr[s.n];
  s.hcon_ptr.assign(nnz + 1, 0);
  for (size_t t = 0; t < s.hess_dst.size(); ++t) s.hcon_ptr[s.hess_dst[t] + 1]++;
  for (int i = 0; i < nnz; ++i) s.hcon_ptr[i + 1] += s.hcon_ptr[i];
  s.hcon_src.resize(s.hess_dst.size());
  {
    std::vector<int32_t> fill(s.hcon_ptr.begin(), s.hcon_ptr.end() - 1);
    for (size_t t = 0; t < s.hess_dst.size(); ++t) s.hcon_src[fill[s.hess_dst[t]]++] = (int32_t)t;
  }
  // force gather (global_composer.hpp:36-66)
  s.fcon_ptr.assign(s.nv + 1, 0);
  for (int t = 0; t < s.nt * cv; ++t) s.fcon_ptr[s.cells[t] + 1]++;
  for (int i = 0; i < s.nv; ++i) s.fcon_ptr[i + 1] += s.fcon_ptr[i];
  s.fcon_src.resize((size_t)s.nt * cv);
  {
    std::vector<int32_t> fill(s.fcon_ptr.begin(), s.fcon_ptr.end() - 1);
    for (int t = 0; t < s.nt * cv; ++t) s.fcon_src[fill[s.cells[t]]++] = t;
  }
}

// boundary_condition::hessian (boundary.hpp:53-67, 96-100): DBC rows/cols -> identity
void filter_dbc_matrix(const orc_ts& s, Vec& vals) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < s.n; ++r)
    for (int k = s.row_ptr[r]; k < s.row_ptr[r + 1]; ++k) {
      const int c = s.col_idx[k];
      if (s.dbc(r) || s.dbc(c)) vals[k] = (r == c) ? 1.0 : 0.0;
    }
}

void spmv(const orc_ts& s, const Vec& vals, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < s.n; ++r) {
    double acc = 0;
    for (int k = s.row_ptr[r]; k < s.row_ptr[r + 1]; ++k) acc += vals[k] * x[s.col_idx[k]];
    y[r] = acc;
  }
}

// deformation_gradient::def_grad_task (def_grad.hpp:93-132): F = Ds * Dminv, x = X + u
void update_def_grad(orc_ts& s, const Vec& u) {
  if (s.springs) return;
  if (s.tri2d) {
    for (int e = 0; e < s.nt; ++e) {
      const int32_t* c = &s.cells[e * 3];
      double x[3][2];
      for (int i = 0; i < 3; ++i)
        for (int d = 0; d < 2; ++d) x[i][d] = s.X[c[i] * 3 + d] + u[c[i] * 3 + d];
      double Ds[4];
      for (int r = 0; r < 2; ++r)
        for (int k = 0; k < 2; ++k) Ds[r * 2 + k] = x[k + 1][r] - x[0][r];
      const double* Dm = &s.dminv[e * 9];
      double* F = &s.defgrad[e * 9];
      for (int r = 0; r < 2; ++r)
        for (int cc = 0; cc < 2; ++cc) F[r * 2 + cc] = Ds[r * 2 + 0] * Dm[0 * 2 + cc] + Ds[r * 2 + 1] * Dm[1 * 2 + cc];
    }
    return;
  }
#pragma omp parallel for schedule(static)
  for (int e = 0; e < s.nt; ++e) {
    const int32_t* c = &s.cells[e * 4];
    double x[4][3];
    for (int i = 0; i < 4; ++i)
      for (int d = 0; d < 3; ++d) x[i][d] = s.X[c[i] * 3 + d] + u[c[i] * 3 + d];
    double Ds[9];
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 3; ++k) Ds[r * 3 + k] = x[k + 1][r] - x[0][r];
    const double* Dm = &s.dminv[e * 9];
    double* F = &s.defgrad[e * 9];
    for (int r = 0; r < 3; ++r)
      for (int cc = 0; cc < 3; ++cc)
        F[r * 3 + cc] = Ds[r * 3 + 0] * Dm[0 * 3 + cc] + Ds[r * 3 + 1] * Dm[1 * 3 + cc] + Ds[r * 3 + 2] * Dm[2 * 3 + cc];
  }
}

// inertia part of update_energy_and_gradients (time_step.hpp:584-592): temp = x - x_inertia,
// f = M temp, E_inertia = 0.5 * temp . f  (unfiltered mass matrix)
double inertia_term(const orc_ts& s, const Vec& u, Vec* f_out) {
  Vec temp(s.n), f(s.n);
  for (int i = 0; i < s.n; ++i) temp[i] = u[i] - s.inertia[i];
  spmv(s, s.mass_vals, temp.data(), f.data());
  const double e = 0.5 * dot(temp, f);
  if (f_out) *f_out = std::move(f);
  return e;
}

// mass-spring elastic part: sum_s k/2 (|x_i - x_j| - L)^2 (times dt^2), edge vectors from differences
// (X_i - X_j) + (u_i - u_j); local forces k (l - L) / l (x_i - x_j) and its negative when lf != null;
// scale = dt^2 sum k/2 (l^2 + L^2)
double spring_energy(const orc_ts& s, const Vec& u, Vec* lf, double* scale) {
  double sum = 0, sc = 0;
  for (int e = 0; e < s.nt; ++e) {
    const int i = s.cells[2 * e], j = s.cells[2 * e + 1];
    double d[3];
    for (int q = 0; q < 3; ++q) d[q] = (s.X[3 * i + q] - s.X[3 * j + q]) + (u[3 * i + q] - u[3 * j + q]);
    const double l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double L = s.sp_rest[e], k = s.sp_k[e], dl = l - L;
    sum += 0.5 * k * dl * dl;
    sc += 0.5 * k * (l * l + L * L);
    if (lf) {
      const double c = l > 0 ? k * dl / l : 0.0;
      for (int q = 0; q < 3; ++q) {
        (*lf)[6 * (size_t)e + q] = c * d[q];
        (*lf)[6 * (size_t)e + 3 + q] = -c * d[q];
      }
    }
  }
  if (scale) *scale = sc * s.dt * s.dt;
  return sum * s.dt * s.dt;
}

double elastic_energy(orc_ts& s, double* scale) {
  double sum = 0, sc = 0;
  if (s.tri2d) {
    for (int e = 0; e < s.nt; ++e) {
      sum += model2_energy(s.model, &s.defgrad[e * 9], s.lam(e), s.mu(e)) * s.vol[e];
      sc += model2_energy_scale(s.model, &s.defgrad[e * 9], s.lam(e), s.mu(e)) * s.vol[e];
    }
    if (scale) *scale = sc * s.dt * s.dt;
    return sum * s.dt * s.dt;
  }
#pragma omp parallel for reduction(+ : sum, sc) schedule(static)
  for (int e = 0; e < s.nt; ++e) {
    sum += model_energy(s.model, &s.defgrad[e * 9], s.lam(e), s.mu(e)) * s.vol[e];
    sc += model_energy_scale(s.model, &s.defgrad[e * 9], s.lam(e), s.mu(e)) * s.vol[e];
  }
  if (scale) *scale = sc * s.dt * s.dt;
  return sum * s.dt * s.dt;
}

double energy_and_gradients(orc_ts& s, bool F_updated) {
  if (s.springs) {
    Vec f;
    const double ei = inertia_term(s, s.next, &f);
    double sc = 0;
    const double ee = spring_energy(s, s.next, &s.local_force, &sc);
    const double a = s.dt * s.dt;
    for (int v = 0; v < s.nv; ++v) {
      double acc[3] = {0, 0, 0};
      for (int k = s.fcon_ptr[v]; k < s.fcon_ptr[v + 1]; ++k)
        for (int d = 0; d < 3; ++d) acc[d] += s.local_force[(size_t)s.fcon_src[k] * 3 + d];
      for (int d = 0; d < 3; ++d) f[v * 3 + d] += a * acc[d];
    }
    for (int i = 0; i < s.n; ++i)
      if (s.dbc(i)) f[i] = 0;
    s.forces = std::move(f);
    s.energy_scale = ei + sc;
    return ei + ee;
  }
  if (!F_updated) update_def_grad(s, s.next);
  Vec f;
  const double inertia_energy = inertia_term(s, s.next, &f);
  // PK1 per element (time_step.hpp:603) and the local-force conversion
  // stress_element_to_vertex (time_step.hpp:62-90): rows 1..3 = (P Dminv^T) columns, row 0 = -sum
  if (s.tri2d) {
    for (int e = 0; e < s.nt; ++e) {
      double P[4];
      s.local_energy[e] = model2_stress(s.model, &s.defgrad[e * 9], s.lam(e), s.mu(e), P);
      const double* Dm = &s.dminv[e * 9];
      double* lf = &s.local_force[e * 9];
      for (int j = 0; j < 3; ++j) lf[0 * 3 + j] = lf[1 * 3 + j] = lf[2 * 3 + j] = 0;
      for (int j = 0; j < 2; ++j) {
        double tot = 0;
        for (int i = 1; i < 3; ++i) {
          const double v = P[j * 2 + 0] * Dm[(i - 1) * 2 + 0] + P[j * 2 + 1] * Dm[(i - 1) * 2 + 1];
          lf[i * 3 + j] = v;
          tot += v;
        }
        lf[0 * 3 + j] = -tot;
      }
    }
  } else
#pragma omp parallel for schedule(static)
  for (int e = 0; e < s.nt; ++e) {
    double P[9];
    s.local_energy[e] = model_stress(s.model, &s.defgrad[e * 9], s.lam(e), s.mu(e), P);
    const double* Dm = &s.dminv[e * 9];
    double* lf = &s.local_force[e * 12];
    for (int j = 0; j < 3; ++j) {
      double tot = 0;
      for (int i = 1; i < 4; ++i) {
        // out = P * Dminv^T, out(j, i-1) = sum_k P(j,k) Dminv(i-1,k)
        const double v = P[j * 3 + 0] * Dm[(i - 1) * 3 + 0] + P[j * 3 + 1] * Dm[(i - 1) * 3 + 1] +
                         P[j * 3 + 2] * Dm[(i - 1) * 3 + 2];
        lf[i * 3 + j] = v;
        tot += v;
      }
      lf[0 * 3 + j] = -tot;
    }
  }
  // gather (time_step.hpp:608-613): f[v] += dt^2 * sum V_e * local_force
  const double a = s.dt * s.dt;
#pragma omp parallel for schedule(static)
  for (int v = 0; v < s.nv; ++v) {
    double acc[3] = {0, 0, 0};
    for (int k = s.fcon_ptr[v]; k < s.fcon_ptr[v + 1]; ++k) {
      const int t = s.fcon_src[k];
      const int e = t / s.cv;
      for (int d = 0; d < 3; ++d) acc[d] += s.vol[e] * s.local_force[t * 3 + d];
    }
    for (int d = 0; d < 3; ++d) f[v * 3 + d] += a * acc[d];
  }
  // boundary_condition::grads (boundary.hpp:45-51)
  for (int i = 0; i < s.n; ++i)
    if (s.dbc(i)) f[i] = 0;
  s.forces = std::move(f);
  double elast = 0, sc = 0;
  for (int e = 0; e < s.nt; ++e) {
    elast += s.local_energy[e] * s.vol[e];
    sc += (s.tri2d ? model2_energy_scale(s.model, &s.defgrad[e * 9], s.lam(e), s.mu(e))
                   : model_energy_scale(s.model, &s.defgrad[e * 9], s.lam(e), s.mu(e))) *
          s.vol[e];
  }
  s.energy_scale = inertia_energy + sc * s.dt * s.dt;
  return inertia_energy + elast * s.dt * s.dt;
}

double energy_only(orc_ts& s, const Vec& u) {
  if (s.springs) return inertia_term(s, u, nullptr) + spring_energy(s, u, nullptr, nullptr);
  update_def_grad(s, u);
  const double ei = inertia_term(s, u, nullptr);
  return ei + elastic_energy(s, nullptr);
}

// update_hessian (time_step.hpp:626-658)
void update_hessian(orc_ts& s, bool F_updated, bool make_spsd, bool filter) {
  if (s.springs) {
    // spring blocks [K, -K; -K, K], K = k [n n^T + c (I - n n^T)], c = 1 - L / l (>= 0 when make_spsd)
    for (int e = 0; e < s.nt; ++e) {
      const int i = s.cells[2 * e], j = s.cells[2 * e + 1];
      double d[3];
      for (int q = 0; q < 3; ++q) d[q] = (s.X[3 * i + q] - s.X[3 * j + q]) + (s.next[3 * i + q] - s.next[3 * j + q]);
      const double l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      double c = l > 0 ? 1.0 - s.sp_rest[e] / l : 0.0;
      if (make_spsd) c = std::max(c, 0.0);
      double nn[3] = {0, 0, 0};
      if (l > 0)
        for (int q = 0; q < 3; ++q) nn[q] = d[q] / l;
      double* K = &s.local_K[(size_t)e * 36];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          const double v = s.sp_k[e] * ((1.0 - c) * nn[a] * nn[b] + (a == b ? c : 0.0));
          K[a * 6 + b] = v;
          K[(3 + a) * 6 + 3 + b] = v;
          K[a * 6 + 3 + b] = -v;
          K[(3 + a) * 6 + b] = -v;
        }
    }
    const double a = s.dt * s.dt;
    const int nnz = (int)s.col_idx.size();
    for (int k = 0; k < nnz; ++k) {
      double acc = 0;
      for (int q = s.hcon_ptr[k]; q < s.hcon_ptr[k + 1]; ++q) acc += s.local_K[s.hcon_src[q]];
      s.sys_vals[k] = s.mass_vals[k] + a * acc;
    }
    if (filter) filter_dbc_matrix(s, s.sys_vals);
    return;
  }
  if (!F_updated) update_def_grad(s, s.next);
  const int LL = 9 * s.cv * s.cv;
  if (s.tri2d) {
    for (int e = 0; e < s.nt; ++e)
      element_stiffness_2d(&s.defgrad[e * 9], &s.dminv[e * 9], s.lam(e), s.mu(e), make_spsd,
                           &s.local_K[(size_t)e * LL], s.model);
  } else {
#pragma omp parallel for schedule(dynamic, 256)
    for (int e = 0; e < s.nt; ++e)
      element_stiffness(&s.defgrad[e * 9], &s.dminv[e * 9], s.lam(e), s.mu(e), make_spsd,
                        &s.local_K[(size_t)e * 144], s.model);
  }
  const double a = s.dt * s.dt;
  const int nnz = (int)s.col_idx.size();
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nnz; ++k) {
    double acc = 0;
    for (int q = s.hcon_ptr[k]; q < s.hcon_ptr[k + 1]; ++q) {
      const int t = s.hcon_src[q];
      acc += s.vol[t / LL] * s.local_K[t];
    }
    s.sys_vals[k] = s.mass_vals[k] + a * acc;
  }
  if (filter) filter_dbc_matrix(s, s.sys_vals);
}

// Jacobi-preconditioned CG (mathprim cg + diagonal_preconditioner, restated as the textbook
// algorithm; x is the initial guess and the result).  Stop: |r| <= rtol*|b|.
int pcg(const orc_ts& s, const Vec& vals, const double* b, double* x, double rtol, int max_iters, int precond,
        double* rel_res) {
  const int n = s.n;
  Vec r(n), z(n), p(n), q(n);
  // preconditioner as one 3x3 block per vertex: 0 identity, 1 Jacobi (diagonal), 2 block-Jacobi
  Vec P(9 * (size_t)s.nv, 0.0);
  for (int u = 0; u < s.nv; ++u) {
    double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 3; ++i)
      for (int k = s.row_ptr[3 * u + i]; k < s.row_ptr[3 * u + i + 1]; ++k) {
        const int c = s.col_idx[k];
        if (c >= 3 * u && c < 3 * u + 3) a[i * 3 + (c - 3 * u)] = vals[k];
      }
    double* m = &P[9 * (size_t)u];
    int mode = precond;
    if (mode == 2) {
      const double det = det3(a);
      if (det > 0 && std::isfinite(det)) {
        inv3(a, m);
        const double m01 = 0.5 * (m[1] + m[3]), m02 = 0.5 * (m[2] + m[6]), m12 = 0.5 * (m[5] + m[7]);
        m[1] = m[3] = m01;
        m[2] = m[6] = m02;
        m[5] = m[7] = m12;
      } else {
        mode = 1;
      }
    }
    if (mode == 1) {
      for (int i = 0; i < 3; ++i) m[i * 4] = a[i * 4] != 0.0 ? 1.0 / a[i * 4] : 1.0;
    } else if (mode == 0) {
      for (int i = 0; i < 3; ++i) m[i * 4] = 1.0;
    }
  }
  auto apply = [&](const Vec& in, Vec& out) {
#pragma omp parallel for schedule(static)
    for (int u = 0; u < s.nv; ++u) {
      const double* m = &P[9 * (size_t)u];
      for (int i = 0; i < 3; ++i)
        out[3 * u + i] = m[i * 3] * in[3 * u] + m[i * 3 + 1] * in[3 * u + 1] + m[i * 3 + 2] * in[3 * u + 2];
    }
  };
  spmv(s, vals, x, q.data());
  for (int i = 0; i < n; ++i) r[i] = b[i] - q[i];
  Vec bv(b, b + n);
  const double bn = nrm2(bv);
  if (bn == 0.0) {
    if (rel_res) *rel_res = 0;
    return 0;
  }
  apply(r, z);
  p = z;
  double rz = dot(r, z);
  int k = 0;
  double rn = nrm2(r);
  for (; k < max_iters; ++k) {
    if (rn <= rtol * bn) break;
    spmv(s, vals, p.data(), q.data());
    const double pq = dot(p, q);
    if (pq <= 0) break;
    const double alpha = rz / pq;
    for (int i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
    }
    apply(r, z);
    const double rr = dot(r, r), rzn = dot(r, z);
    rn = std::sqrt(rr);
    const double beta = rzn / rz;
    rz = rzn;
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
  }
  if (rel_res) *rel_res = rn / bn;
  return k;
}

// mass_integrator / laplace_integrator (bilinears.hpp:132-167, 191-264) for one tet
void element_mass(const double* Xv[4], double rho, double M[16]) {
  double J[9];
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) J[r * 3 + k] = Xv[k + 1][r] - Xv[0][r];
  const double detJ = std::fabs(det3(J));
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) M[i * 4 + j] = (detJ * (i == j ? 1.0 / 60 : 1.0 / 120)) * rho;
}

void element_laplace(const double* Xv[4], double alpha, double L[16]) {
  double J[9], iJ[9];
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) J[r * 3 + k] = Xv[k + 1][r] - Xv[0][r];
  const double detJ = std::fabs(det3(J));
  inv3(J, iJ);
  // grad phi_i (i>=1) = row i-1 of J^{-1}; grad phi_0 = -sum.  integral = |det J|/6 * gi.gj
  double g[4][3];
  for (int k = 0; k < 3; ++k) {
    g[1][k] = iJ[0 * 3 + k];
    g[2][k] = iJ[1 * 3 + k];
    g[3][k] = iJ[2 * 3 + k];
    g[0][k] = -(g[1][k] + g[2][k] + g[3][k]);
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      L[i * 4 + j] = alpha * detJ / 6.0 * (g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2]);
}

bool stop_ok(const orc_ts& s, const orc_params& p, double gn, double g0) {
  if (p.stop_mode == 0) return gn < s.abs_tol;
  // the absolute rule at rtol = stop_floor as a floor (a step from rest has a round-off gradient)
  return gn <= p.rel_tol * g0 || gn <= p.stop_floor * s.mass_third;
}

}  // namespace

// ===========================================================================
// C API
// ===========================================================================
extern "C" {

int orc_unit_box_sizes(int nx, int ny, int nz, int* nv, int* nt) {
  *nv = nx * ny * nz;
  *nt = 5 * (nx - 1) * (ny - 1) * (nz - 1);
  return 0;
}

// ssim::mesh::unit_box (common_shapes.hpp:67-132)
void orc_unit_box(int nx, int ny, int nz, double* X, int32_t* cells) {
  int id = 0;
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k < nz; ++k) {
        X[id * 3 + 0] = i / double(nx - 1);
        X[id * 3 + 1] = j / double(ny - 1);
        X[id * 3 + 2] = k / double(nz - 1);
        ++id;
      }
  id = 0;
  for (int i = 0; i < nx - 1; ++i)
    for (int j = 0; j < ny - 1; ++j)
      for (int k = 0; k < nz - 1; ++k) {
        int v000 = i * ny * nz + j * nz + k, v100 = (i + 1) * ny * nz + j * nz + k;
        int v010 = i * ny * nz + (j + 1) * nz + k, v001 = i * ny * nz + j * nz + k + 1;
        int v110 = (i + 1) * ny * nz + (j + 1) * nz + k, v101 = (i + 1) * ny * nz + j * nz + k + 1;
        int v011 = i * ny * nz + (j + 1) * nz + k + 1, v111 = (i + 1) * ny * nz + (j + 1) * nz + k + 1;
        if (i % 2 == 1) {
          std::swap(v000, v100);
          std::swap(v010, v110);
          std::swap(v001, v101);
          std::swap(v011, v111);
        }
        if (j % 2 == 1) {
          std::swap(v000, v010);
          std::swap(v100, v110);
          std::swap(v001, v011);
          std::swap(v101, v111);
        }
        if (k % 2 == 1) {
          std::swap(v000, v001);
          std::swap(v100, v101);
          std::swap(v010, v011);
          std::swap(v110, v111);
        }
        const int t[5][4] = {{v000, v100, v010, v001},
                             {v010, v100, v110, v111},
                             {v100, v010, v001, v111},
                             {v100, v001, v101, v111},
                             {v011, v001, v010, v111}};
        for (int q = 0; q < 5; ++q) {
          for (int c = 0; c < 4; ++c) cells[id * 4 + c] = t[q][c];
          ++id;
        }
      }
}

// ssim::mesh::tetra (common_shapes.hpp:134-145)
void orc_tetra(double* X, int32_t* cells) {
  const double v[12] = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
  std::memcpy(X, v, sizeof(v));
  for (int i = 0; i < 4; ++i) cells[i] = i;
}

void orc_lame(double E, double nu, double* lambda, double* mu) {
  *mu = E / (2 * (1 + nu));
  *lambda = E * nu / ((1 + nu) * (1 - 2 * nu));
}
double orc_snh_energy(const double F[9], double lambda, double mu) { return snh_energy(F, lambda, mu); }
double orc_snh2_energy(const double F[4], double lambda, double mu) { return snh2_energy(F, lambda, mu); }
double orc_snh2_stress(const double F[4], double lambda, double mu, double P[4]) {
  return snh2_stress(F, lambda, mu, P);
}
void orc_snh2_hessian(const double F[4], double lambda, double mu, double H[16]) { snh2_hessian(F, lambda, mu, H); }
double orc_linear2_stress(const double F[4], double lambda, double mu, double P[4]) {
  return linear2_stress(F, lambda, mu, P);
}
void orc_linear2_hessian(double lambda, double mu, double H[16]) { linear2_hessian(lambda, mu, H); }
void orc_element_stiffness_2d(const double F[4], const double Dminv[4], double lambda, double mu, int make_spsd,
                              int model, double K[81]) {
  element_stiffness_2d(F, Dminv, lambda, mu, make_spsd != 0, K, model);
}
double orc_snh_stress(const double F[9], double lambda, double mu, double P[9]) {
  return snh_stress(F, lambda, mu, P);
}
void orc_snh_hessian(const double F[9], double lambda, double mu, double H[81]) { snh_hessian(F, lambda, mu, H); }
int orc_sym_eigen(int n, const double* A, double* evals, double* evecs) { return sym_eigen(n, A, evals, evecs); }
void orc_project_spd(const double H[81], double eps, double Hp[81]) { project_spd(H, eps, Hp); }

// dminv_task (def_grad.hpp:56-91) and rest_vol_task (rest_vol.hpp:34-54)
void orc_dminv(const double x0[3], const double x1[3], const double x2[3], const double x3[3], double Dminv[9],
               double* vol) {
  double Dm[9];
  for (int r = 0; r < 3; ++r) {
    Dm[r * 3 + 0] = x1[r] - x0[r];
    Dm[r * 3 + 1] = x2[r] - x0[r];
    Dm[r * 3 + 2] = x3[r] - x0[r];
  }
  inv3(Dm, Dminv);
  if (vol) *vol = std::fabs(det3(Dm) / 6);
}

void orc_element_stiffness(const double F[9], const double Dminv[9], double lambda, double mu, int make_spsd,
                           double K[144]) {
  element_stiffness(F, Dminv, lambda, mu, make_spsd != 0, K);
}

void orc_default_params(orc_params* p) {
  p->max_newton_iters = 1000;
  p->armijo = 0.3;
  p->ls_shrink = 0.5;
  p->max_ls_iters = 30;
  p->cg_max_iters = 10000;
  p->cg_rtol = 1e-8;
  p->cg_forcing = 0;
  p->cg_eta_min = 1e-6;
  p->stop_mode = 0;
  p->rel_tol = 1e-6;
  p->precond = 1;
  p->lbfgs_history = 8;
  p->lbfgs_armijo = 1e-4;
  p->max_lbfgs_iters = 1000;
  p->ls_energy_slack = 1e-14;
  p->ncg_max_iters = 1000;
  p->ncg_step0 = 1e-2;
  p->ncg_eta = 0.5;
  p->ncg_expand = 3;
  p->stop_floor = 1e-12;
}

orc_ts* orc_create(const double* X, int nv, const int32_t* cells, int nt, double dt, double E, double nu,
                   double rho) {
  orc_ts* s = new orc_ts;
  s->nv = nv;
  s->nt = nt;
  s->n = nv * 3;
  s->X.assign(X, X + (size_t)nv * 3);
  s->cells.assign(cells, cells + (size_t)nt * 4);
  s->dt = dt;
  s->E = E;
  s->nu = nu;
  s->rho = rho;
  s->dof_type.assign(s->n, 0);
  for (Vec* v : {&s->dbc_values, &s->deformation, &s->prev_deform, &s->inertia, &s->next, &s->velocity,
                 &s->ext_accel, &s->forces})
    v->assign(s->n, 0.0);
  orc_reset(s);  // the constructor calls reset() (time_step.hpp:260-265)
  return s;
}

orc_ts* orc_create_2d(const double* X2, int nv, const int32_t* tris, int nt, double dt, double E, double nu,
                      double rho) {
  orc_ts* s = new orc_ts;
  s->tri2d = true;
  s->cv = 3;
  s->nv = nv;
  s->nt = nt;
  s->n = nv * 3;
  s->X.assign((size_t)nv * 3, 0.0);
  for (int v = 0; v < nv; ++v) {
    s->X[3 * v] = X2[2 * v];
    s->X[3 * v + 1] = X2[2 * v + 1];
  }
  s->cells.assign(tris, tris + (size_t)nt * 3);
  s->dt = dt;
  s->E = E;
  s->nu = nu;
  s->rho = rho;
  s->dof_type.assign(s->n, 0);
  for (Vec* v : {&s->dbc_values, &s->deformation, &s->prev_deform, &s->inertia, &s->next, &s->velocity,
                 &s->ext_accel, &s->forces})
    v->assign(s->n, 0.0);
  orc_reset(s);
  return s;
}

orc_ts* orc_create_springs(const double* X, int nv, const int32_t* springs, int ns, double k, const double* vmass,
                           double m, double dt) {
  orc_ts* s = new orc_ts;
  s->springs = true;
  s->cv = 2;
  s->nv = nv;
  s->nt = ns;
  s->n = nv * 3;
  s->X.assign(X, X + (size_t)nv * 3);
  s->cells.assign(springs, springs + (size_t)ns * 2);
  s->dt = dt;
  s->E = 1.0;
  s->nu = 0.25;
  s->rho = 0.0;
  s->sp_rest.assign(ns, 0.0);
  for (int e = 0; e < ns; ++e) {
    const int i = springs[2 * e], j = springs[2 * e + 1];
    double l2 = 0;
    for (int q = 0; q < 3; ++q) l2 += (X[3 * i + q] - X[3 * j + q]) * (X[3 * i + q] - X[3 * j + q]);
    s->sp_rest[e] = std::sqrt(l2);
  }
  s->sp_k.assign(ns, k);
  if (vmass)
    s->vmass.assign(vmass, vmass + nv);
  else
    s->vmass.assign(nv, m);
  s->dof_type.assign(s->n, 0);
  for (Vec* v : {&s->dbc_values, &s->deformation, &s->prev_deform, &s->inertia, &s->next, &s->velocity,
                 &s->ext_accel, &s->forces})
    v->assign(s->n, 0.0);
  orc_reset(s);
  return s;
}

void orc_destroy(orc_ts* s) { delete s; }
int orc_num_vertices(const orc_ts* s) { return s->nv; }
int orc_num_cells(const orc_ts* s) { return s->nt; }
int orc_nnz(const orc_ts* s) { return (int)s->col_idx.size(); }
double orc_threshold_abs(const orc_ts* s) { return s->abs_tol; }

int orc_set_time_step(orc_ts* s, double dt) {
  if (!(dt > 0)) return -1;
  s->dt = dt;
  return 0;
}
int orc_set_youngs(orc_ts* s, double E) {
  if (!(E > 0)) return -1;
  s->E = E;
  return 0;
}
int orc_set_poisson(orc_ts* s, double nu) {
  if (!(nu > 0 && nu < 0.5)) return -1;
  s->nu = nu;
  return 0;
}
int orc_set_density(orc_ts* s, double rho) {
  if (!(rho > 0)) return -1;
  s->rho = rho;
  return 0;
}
int orc_set_damping(orc_ts* s, double d) {
  if (!(0 <= d && d < 1)) return -1;
  s->damping = d;
  return 0;
}
int orc_set_threshold(orc_ts* s, double r) {
  if (!(0 < r && r < 1)) return -1;
  s->rtol = r;
  return 0;
}
void orc_set_material(orc_ts* s, const double* Ee, const double* ne) {
  if (Ee)
    s->E_elem.assign(Ee, Ee + s->nt);
  else
    s->E_elem.clear();
  if (ne)
    s->nu_elem.assign(ne, ne + s->nt);
  else
    s->nu_elem.clear();
}
void orc_set_dof_type(orc_ts* s, const int8_t* t) { s->dof_type.assign(t, t + s->n); }
void orc_get_dof_type(const orc_ts* s, int8_t* t) { std::copy(s->dof_type.begin(), s->dof_type.end(), t); }
void orc_set_pd_diffusivity_mode(orc_ts* s, int mode) { s->pd_diff_mode = mode; }

// add_ext_force_dof (time_step.hpp:550-557)
int orc_add_ext_force_dof(orc_ts* s, int dof, double a) {
  if (!(-3 < dof && dof < 3)) return -1;
  if (dof < 0) dof += 3;
  for (int v = 0; v < s->nv; ++v) s->ext_accel[v * 3 + dof] += a;
  return 0;
}

// reset (time_step.hpp:363-494)
void orc_reset(orc_ts* s) {
  if (s->springs) {
    s->local_force.assign((size_t)s->nt * 6, 0);
    s->local_K.assign((size_t)s->nt * 36, 0);
    for (Vec* v : {&s->inertia, &s->next, &s->forces}) v->assign(s->n, 0.0);
    build_pattern(*s);
    const int nnz = (int)s->col_idx.size();
    s->mass_vals.assign(nnz, 0.0);  // lumped: m_v on the dof diagonals
    for (int r = 0; r < s->n; ++r)
      for (int k = s->row_ptr[r]; k < s->row_ptr[r + 1]; ++k)
        if (s->col_idx[k] == r) s->mass_vals[k] = s->vmass[r / 3];
    s->massf_vals = s->mass_vals;
    filter_dbc_matrix(*s, s->massf_vals);
    s->sys_vals = s->mass_vals;
    double asum = 0;
    for (double v : s->mass_vals) asum += std::fabs(v);
    s->abs_tol = asum / 3.0 * s->rtol;
    s->mass_third = asum / 3.0;
    s->has_reset = true;
    s->pd_ready = false;
    return;
  }
  if (s->tri2d) {
    // rest shape (def_grad.hpp:56-91, rest_vol.hpp:34-54 with PhysicalDim 2): Dm^-1 (row-major 2x2 in the
    // first 4 of 9 slots), area |det Dm| / 2; consistent mass from p1_element_2d
    s->dminv.assign((size_t)s->nt * 9, 0);
    s->vol.assign(s->nt, 0);
    s->defgrad.assign((size_t)s->nt * 9, 0);
    s->local_energy.assign(s->nt, 0);
    s->local_force.assign((size_t)s->nt * 9, 0);
    s->local_K.assign((size_t)s->nt * 81, 0);
    for (Vec* v : {&s->inertia, &s->next, &s->forces}) v->assign(s->n, 0.0);
    for (int e = 0; e < s->nt; ++e) {
      const int32_t* c = &s->cells[e * 3];
      const double D[4] = {s->X[c[1] * 3] - s->X[c[0] * 3], s->X[c[2] * 3] - s->X[c[0] * 3],
                           s->X[c[1] * 3 + 1] - s->X[c[0] * 3 + 1], s->X[c[2] * 3 + 1] - s->X[c[0] * 3 + 1]};
      const double det = D[0] * D[3] - D[1] * D[2];
      double* Dm = &s->dminv[e * 9];
      Dm[0] = D[3] / det;
      Dm[1] = -D[1] / det;
      Dm[2] = -D[2] / det;
      Dm[3] = D[0] / det;
      s->vol[e] = std::fabs(det / 2);
    }
    build_pattern(*s);
    const int nnz = (int)s->col_idx.size();
    s->mass_vals.assign(nnz, 0.0);
    for (int e = 0; e < s->nt; ++e) {
      const int32_t* c = &s->cells[e * 3];
      const double* Xv[3] = {&s->X[c[0] * 3], &s->X[c[1] * 3], &s->X[c[2] * 3]};
      double M[9];
      element_mass_2d(Xv, s->rho, M);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          for (int a = 0; a < 3; ++a) s->mass_vals[s->hess_dst[(size_t)e * 81 + (i * 3 + a) * 9 + j * 3 + a]] += M[i * 3 + j];
    }
    s->massf_vals = s->mass_vals;
    filter_dbc_matrix(*s, s->massf_vals);
    s->sys_vals = s->mass_vals;
    double asum = 0;  // asum(mass) / dofs_per_node (time_step.hpp:490): the z copies add 1/3 of it
    for (double v : s->mass_vals) asum += std::fabs(v);
    s->abs_tol = asum / 3.0 * s->rtol;
    s->mass_third = asum / 3.0;
    s->has_reset = true;
    s->pd_ready = false;
    return;
  }
  s->dminv.assign((size_t)s->nt * 9, 0);
  s->vol.assign(s->nt, 0);
  s->defgrad.assign((size_t)s->nt * 9, 0);
  s->local_energy.assign(s->nt, 0);
  s->local_force.assign((size_t)s->nt * 12, 0);
  s->local_K.assign((size_t)s->nt * 144, 0);
  for (Vec* v : {&s->inertia, &s->next, &s->forces}) v->assign(s->n, 0.0);
#pragma omp parallel for schedule(static)
  for (int e = 0; e < s->nt; ++e) {
    const int32_t* c = &s->cells[e * 4];
    orc_dminv(&s->X[c[0] * 3], &s->X[c[1] * 3], &s->X[c[2] * 3], &s->X[c[3] * 3], &s->dminv[e * 9], &s->vol[e]);
  }
  build_pattern(*s);
  const int nnz = (int)s->col_idx.size();
  // consistent mass (time_step.hpp:437-461): triplets over (i, j, a, b), value only for a == b
  s->mass_vals.assign(nnz, 0.0);
  for (int e = 0; e < s->nt; ++e) {
    const int32_t* c = &s->cells[e * 4];
    const double* Xv[4] = {&s->X[c[0] * 3], &s->X[c[1] * 3], &s->X[c[2] * 3], &s->X[c[3] * 3]};
    double M[16];
    element_mass(Xv, s->rho, M);
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        for (int a = 0; a < 3; ++a) s->mass_vals[s->hess_dst[(size_t)e * 144 + (i * 3 + a) * 12 + j * 3 + a]] += M[i * 4 + j];
  }
  s->massf_vals = s->mass_vals;
  filter_dbc_matrix(*s, s->massf_vals);
  s->sys_vals = s->mass_vals;
  // convergence threshold (time_step.hpp:490-491): rtol * asum(mass values) / 3
  double asum = 0;
  for (double v : s->mass_vals) asum += std::fabs(v);
  s->abs_tol = asum / 3.0 * s->rtol;
  s->mass_third = asum / 3.0;
  s->has_reset = true;
  s->pd_ready = false;
}

// prepare_step (time_step.hpp:499-518)
void orc_prepare_step(orc_ts* s) {
  for (int i = 0; i < s->n; ++i)
    s->inertia[i] = s->deformation[i] + s->dt * s->velocity[i] + s->dt * s->dt * s->ext_accel[i];
  for (int i = 0; i < s->n; ++i)
    if (s->dbc(i)) s->inertia[i] = s->dbc_values[i];
  s->next = s->inertia;
}

double orc_update_energy_and_gradients(orc_ts* s, int F_updated) { return energy_and_gradients(*s, F_updated != 0); }

double orc_energy_at(orc_ts* s, const double* u) {
  Vec uu(u, u + s->n);
  return energy_only(*s, uu);
}

void orc_update_hessian(orc_ts* s, int F_updated, int make_spsd, int filter_dbc) {
  update_hessian(*s, F_updated != 0, make_spsd != 0, filter_dbc != 0);
}

// Newton stepper: time_step_solver_backward_euler::solve_impl (backward_euler.hpp:15-33) driving
// mathprim's newton_optimizer (not in the reference tree; definition restated here):
//   loop: evaluate E, g; stop if the gradient test passes; H = update_hessian(true, make_spsd=true)
//   (variational_problem::eval_hessian_impl, time_step.hpp:764-768); d from Jacobi-PCG on H d = -g;
//   backtracking line search from alpha = 1, shrink `ls_shrink`, Armijo constant `armijo`, accepting
//   E(x + a d) <= E + armijo a g.d + ls_energy_slack S_E, with S_E the sum of the magnitudes of the
//   energy's terms (the scale of its round-off: without the slack the test cannot pass once the Newton
//   decrement falls below that floor); x += a d.
// Then compute_step (time_step.hpp:520-528) re-evaluates the gradient and returns its norm.
double orc_compute_step_newton(orc_ts* s, const orc_params* p, orc_stats* st) {
  orc_stats loc{};
  double E = energy_and_gradients(*s, false);
  const double g0 = nrm2(s->forces);
  loc.grad_norm0 = g0;
  Vec d(s->n), xt(s->n), b(s->n);
  int it = 0;
  for (;; ++it) {
    const double gn = nrm2(s->forces);
    loc.grad_norm = gn;
    loc.energy = E;
    if (stop_ok(*s, *p, gn, g0)) {
      loc.converged = 1;
      break;
    }
    if (it >= p->max_newton_iters) break;
    update_hessian(*s, true, true, true);
    double eta = p->cg_rtol;
    if (p->cg_forcing == 1 && g0 > 0) eta = std::min(p->cg_rtol, std::max(p->cg_eta_min, gn / g0));
    for (int i = 0; i < s->n; ++i) {
      b[i] = -s->forces[i];
      d[i] = 0;
    }
    double rr;
    loc.cg_iters_total += pcg(*s, s->sys_vals, b.data(), d.data(), eta, p->cg_max_iters, p->precond, &rr);
    double gd = dot(s->forces, d);
    if (!(gd < 0)) {  // not a descent direction: fall back to steepest descent
      for (int i = 0; i < s->n; ++i) d[i] = -s->forces[i];
      gd = -gn * gn;
    }
    double alpha = 1.0;
    const double Escale = s->energy_scale;
    for (int ls = 0; ls < p->max_ls_iters; ++ls) {
      for (int i = 0; i < s->n; ++i) xt[i] = s->next[i] + alpha * d[i];
      const double Et = energy_only(*s, xt);
      loc.ls_steps_total++;
      if (Et <= E + p->armijo * alpha * gd + p->ls_energy_slack * Escale) break;
      alpha *= p->ls_shrink;
    }
    double ch = 0;
    for (int i = 0; i < s->n; ++i) {
      s->next[i] += alpha * d[i];
      ch = std::max(ch, std::fabs(alpha * d[i]));
    }
    loc.last_change = ch;
    E = energy_and_gradients(*s, false);
  }
  loc.newton_iters = it;
  if (st) *st = loc;
  energy_and_gradients(*s, false);
  return nrm2(s->forces);
}

// L-BFGS stepper (backward_euler.hpp:43-67) over mathprim's l_bfgs_optimizer (restated here as the
// two-loop recursion of Nocedal & Wright, Alg. 7.4, with backtracking Armijo line search).  When
// `Ainv` is set, the initial inverse Hessian is that solve (projective_dynamics.hpp:31-34).
// mode: 0 plain L-BFGS, 1 PD (initial inverse Hessian = PD matrix solve), 2 H0 (= solve with the projected
// Hessian at the start of the step, time_step_solver_h0, projective_dynamics.hpp:100-150)
static double lbfgs_core(orc_ts* s, const orc_params* p, orc_stats* st, int mode) {
  const bool pd = mode != 0;
  Vec h0_vals;
  if (mode == 2) {
    update_hessian(*s, false, true, true);  // s.update_hessian(false, true) at the step start
    h0_vals = s->sys_vals;
  }
  orc_stats loc{};
  const int n = s->n, m = std::max(1, p->lbfgs_history);
  std::vector<Vec> S, Y;
  std::vector<double> rho;
  double E = energy_and_gradients(*s, false);
  Vec g = s->forces;
  const double g0 = nrm2(g);
  loc.grad_norm0 = g0;
  Vec q(n), z(n), xt(n);
  int it = 0;
  for (;; ++it) {
    const double gn = nrm2(g);
    loc.grad_norm = gn;
    loc.energy = E;
    if (stop_ok(*s, *p, gn, g0)) {
      loc.converged = 1;
      break;
    }
    if (it >= p->max_lbfgs_iters) break;
    q = g;
    const int h = (int)S.size();
    std::vector<double> al(h);
    for (int i = h - 1; i >= 0; --i) {
      al[i] = rho[i] * dot(S[i], q);
      for (int k = 0; k < n; ++k) q[k] -= al[i] * Y[i][k];
    }
    if (pd) {
      std::fill(z.begin(), z.end(), 0.0);
      double rr;
      pcg(*s, mode == 2 ? h0_vals : s->pd_vals, q.data(), z.data(), 1e-12, 100000, 1, &rr);
    } else {
      double gamma = 1.0 / std::max(gn, 1e-300);
      if (h > 0) gamma = dot(S[h - 1], Y[h - 1]) / dot(Y[h - 1], Y[h - 1]);
      for (int k = 0; k < n; ++k) z[k] = gamma * q[k];
    }
    for (int i = 0; i < h; ++i) {
      const double bb = rho[i] * dot(Y[i], z);
      for (int k = 0; k < n; ++k) z[k] += S[i][k] * (al[i] - bb);
    }
    for (int k = 0; k < n; ++k) z[k] = -z[k];
    double gd = dot(g, z);
    if (!(gd < 0)) {
      S.clear();
      Y.clear();
      rho.clear();
      for (int k = 0; k < n; ++k) z[k] = -g[k] / std::max(gn, 1e-300);
      gd = dot(g, z);
    }
    double alpha = 1.0;
    const double Escale = s->energy_scale;
    for (int ls = 0; ls < p->max_ls_iters; ++ls) {
      for (int k = 0; k < n; ++k) xt[k] = s->next[k] + alpha * z[k];
      const double Et = energy_only(*s, xt);
      loc.ls_steps_total++;
      if (Et <= E + p->lbfgs_armijo * alpha * gd + p->ls_energy_slack * Escale) break;
      alpha *= p->ls_shrink;
    }
    Vec sv(n), yv(n);
    for (int k = 0; k < n; ++k) {
      sv[k] = alpha * z[k];
      s->next[k] += sv[k];
    }
    E = energy_and_gradients(*s, false);
    for (int k = 0; k < n; ++k) yv[k] = s->forces[k] - g[k];
    g = s->forces;
    const double sy = dot(sv, yv);
    if (sy > 1e-300) {
      if ((int)S.size() == m) {
        S.erase(S.begin());
        Y.erase(Y.begin());
        rho.erase(rho.begin());
      }
      S.push_back(std::move(sv));
      Y.push_back(std::move(yv));
      rho.push_back(1.0 / sy);
    }
  }
  loc.newton_iters = it;
  if (st) *st = loc;
  energy_and_gradients(*s, false);
  return nrm2(s->forces);
}

// ---------------------------------------------------------------- nonlinear CG
// Reference: time_step_solver_ncg / _with_ext_prec (nonlinear_cg.hpp:9-97) run mathprim's ncg_optimizer
// with the Dai-Kou strategy, a backtracking line search, learning rate 1e-2 and at most 1000 iterations;
// the preconditioned variant applies x = L (L^T g) (nonlinear_cg.hpp:52-57).  mathprim is not in the
// reference tree, so the iteration is restated from the published method and is parity-unpinned:
//   direction: d0 = -H g0 (H = L L^T, identity by default); d_{k+1} = -H g_{k+1} + beta d_k with the
//     Dai-Kou beta (Y.-H. Dai, C.-X. Kou, SIAM J. Optim. 23(1) 2013, tau_k = s^T y / |s|^2):
//     beta = g^T H y / d^T y - (y^T H y) (g^T d) / (d^T y)^2, truncated to >= eta g^T d / |d|^2
//     (g the new gradient, d the last direction, y = g_new - g_old); restart d = -H g when not descending;
//   line search: Armijo (lbfgs_armijo) backtracking from alpha_init, a failed trial shrinks to the
//     minimiser of the parabola through E, g^T d and the trial energy, clamped to [0.1, 0.5] alpha; after
//     an accepted trial, up to ncg_expand moves to that parabola's minimiser when it lies beyond 1.5
//     alpha (at most 10 alpha), kept while the energy decreases;
//   alpha_init(0) = ncg_step0, alpha_init(k) = alpha(k-1) (g_{k-1}^T d_{k-1}) / (g_k^T d_k).
static void ncg_apply(const orc_ts& s, bool prec, const Vec& g, Vec& z) {
  const int n = s.n;
  if (!prec || s.ncg_L.empty()) {
    z = g;
    return;
  }
  // t = L^T g (row i of L^T = column i of L: read through the transposed entry of the symmetric pattern)
  Vec t(n, 0.0);
  for (int r = 0; r < n; ++r) {
    double acc = 0;
    for (int k = s.row_ptr[r]; k < s.row_ptr[r + 1]; ++k) {
      const int c = s.col_idx[k];
      // L[c][r]: position of r in row c
      const int* b = s.col_idx.data() + s.row_ptr[c];
      const int* e = s.col_idx.data() + s.row_ptr[c + 1];
      const int kt = (int)(std::lower_bound(b, e, r) - s.col_idx.data());
      acc += s.ncg_L[kt] * g[c];
    }
    t[r] = acc;
  }
  z.assign(n, 0.0);
  for (int r = 0; r < n; ++r) {
    double acc = 0;
    for (int k = s.row_ptr[r]; k < s.row_ptr[r + 1]; ++k) acc += s.ncg_L[k] * t[s.col_idx[k]];
    z[r] = acc;
  }
}

static double ncg_core(orc_ts* s, const orc_params* p, orc_stats* st, bool prec) {
  orc_stats loc{};
  const int n = s->n;
  double E = energy_and_gradients(*s, false);
  double Escale = s->energy_scale;
  Vec g = s->forces, gprev = g, z(n), y(n), hy(n), d(n), xt(n);
  const double g0 = nrm2(g);
  loc.grad_norm0 = g0;
  ncg_apply(*s, prec, g, z);
  for (int k = 0; k < n; ++k) d[k] = -z[k];
  double gd = dot(g, d);
  double alpha_init = p->ncg_step0;
  int it = 0;
  auto trial = [&](double a) {
    for (int k = 0; k < n; ++k) xt[k] = s->next[k] + a * d[k];
    loc.ls_steps_total++;
    return energy_only(*s, xt);
  };
  for (;; ++it) {
    const double gn = nrm2(g);
    loc.grad_norm = gn;
    loc.energy = E;
    if (stop_ok(*s, *p, gn, g0)) {
      loc.converged = 1;
      break;
    }
    if (it >= p->ncg_max_iters) break;
    if (!(gd < 0)) {  // restart
      for (int k = 0; k < n; ++k) d[k] = -z[k];
      gd = dot(g, d);
      if (!(gd < 0)) {
        for (int k = 0; k < n; ++k) d[k] = -g[k];
        gd = dot(g, d);
      }
      alpha_init = p->ncg_step0;
    }
    double a = alpha_init, Et = trial(a);
    const double slack = p->ls_energy_slack * Escale;
    auto armijo = [&](double aa, double ee) { return ee <= E + p->lbfgs_armijo * aa * gd + slack; };
    for (int ls = 1; ls < p->max_ls_iters && !armijo(a, Et); ++ls) {
      const double c2 = (Et - E - gd * a) / (a * a);
      double an = c2 > 0 ? -gd / (2 * c2) : 0.5 * a;
      if (!std::isfinite(an)) an = 0.5 * a;
      a = std::min(std::max(an, 0.1 * a), 0.5 * a);
      Et = trial(a);
    }
    for (int ex = 0; ex < p->ncg_expand && armijo(a, Et); ++ex) {
      const double c2 = (Et - E - gd * a) / (a * a);
      if (!(c2 > 0)) break;
      const double astar = -gd / (2 * c2);
      if (!(astar > 1.5 * a)) break;
      const double an = std::min(astar, 10 * a);
      const double En = trial(an);
      if (!(En < Et) || !armijo(an, En)) break;
      a = an;
      Et = En;
    }
    for (int k = 0; k < n; ++k) s->next[k] += a * d[k];
    loc.last_change = a * nrm2(d);
    E = energy_and_gradients(*s, false);
    Escale = s->energy_scale;
    g = s->forces;
    for (int k = 0; k < n; ++k) y[k] = g[k] - gprev[k];
    gprev = g;
    ncg_apply(*s, prec, g, z);
    if (prec && !s->ncg_L.empty())
      ncg_apply(*s, prec, y, hy);
    else
      hy = y;
    const double dy = dot(d, y), zy = dot(z, y), yhy = dot(y, hy), gdn = dot(g, d), dd = dot(d, d);
    double beta = 0;
    if (dy > 1e-300) beta = zy / dy - yhy * gdn / (dy * dy);
    if (dd > 0) beta = std::max(beta, p->ncg_eta * gdn / dd);
    const double gd_old = gd;
    for (int k = 0; k < n; ++k) d[k] = beta * d[k] - z[k];
    gd = dot(g, d);
    alpha_init = (gd < 0 && gd_old < 0) ? a * gd_old / gd : p->ncg_step0;
  }
  loc.newton_iters = it;
  if (st) *st = loc;
  energy_and_gradients(*s, false);
  return nrm2(s->forces);
}

double orc_compute_step_ncg(orc_ts* s, const orc_params* p, orc_stats* st) { return ncg_core(s, p, st, false); }
double orc_compute_step_ncg_prec(orc_ts* s, const orc_params* p, orc_stats* st) { return ncg_core(s, p, st, true); }

void orc_set_model(orc_ts* s, int model) { s->model = model; }

double orc_linear_stress(const double F[9], double lambda, double mu, double P[9]) {
  return linear_stress(F, lambda, mu, P);
}
void orc_linear_hessian(double lambda, double mu, double H[81]) { linear_hessian(lambda, mu, H); }
void orc_element_stiffness_model(const double F[9], const double Dminv[9], double lambda, double mu, int make_spsd,
                                 int model, double K[144]) {
  element_stiffness(F, Dminv, lambda, mu, make_spsd != 0, K, model);
}

void orc_set_ncg_matrix(orc_ts* s, const double* values) {
  if (!values) {
    s->ncg_L.clear();
    return;
  }
  s->ncg_L.assign(values, values + s->col_idx.size());
}

double orc_compute_step_lbfgs(orc_ts* s, const orc_params* p, orc_stats* st) { return lbfgs_core(s, p, st, 0); }

double orc_compute_step_h0(orc_ts* s, const orc_params* p, orc_stats* st) { return lbfgs_core(s, p, st, 2); }

// time_step_solver_forward_euler (time_step.hpp:717-736): evaluate, then next += dt^2/2 * forces (the
// gradient of the incremental potential, as the reference adds it); compute_step then re-evaluates
double orc_compute_step_forward_euler(orc_ts* s, const orc_params*, orc_stats* st) {
  energy_and_gradients(*s, false);
  const double a = 0.5 * s->dt * s->dt;
  for (int i = 0; i < s->n; ++i) s->next[i] += a * s->forces[i];
  const double E = energy_and_gradients(*s, false);
  if (st) {
    *st = orc_stats{};
    st->energy = E;
    st->grad_norm = nrm2(s->forces);
  }
  return nrm2(s->forces);
}

// PD matrix (projective_dynamics.hpp:53-93): (mass(rho) + laplace(dt^2 * kappa)) (x) I3 with the DBC
// identity filter.  kappa = approximated_diffusivity (stable_neohookean.hpp:106-111) of
// uniform_elasticity() (time_step.hpp:356), which constructs the model as ElastModel{E, nu}: the
// model's (lambda, mu) slots then hold (E, nu).  Mode 1 uses the Lame parameters instead, mode 2 each
// element's own Lame parameters (an extension for per-element materials).
void orc_pd_matrix_values(orc_ts* s, double* out) {
  if (s->springs) {
    // mass-spring projective dynamics (Liu et al. 2013): M + dt^2 sum_s k_s (A_s^T A_s) (x) I3
    Vec vals = s->mass_vals;
    for (int e = 0; e < s->nt; ++e) {
      const double w = s->dt * s->dt * s->sp_k[e];
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
          for (int a = 0; a < 3; ++a)
            vals[s->hess_dst[(size_t)e * 36 + (i * 3 + a) * 6 + j * 3 + a]] += (i == j ? w : -w);
    }
    filter_dbc_matrix(*s, vals);
    s->pd_vals = vals;
    s->pd_ready = true;
    if (out) std::copy(vals.begin(), vals.end(), out);
    return;
  }
  double lam_slot = s->E, mu_slot = s->nu;
  if (s->pd_diff_mode == 1) orc_lame(s->E, s->nu, &lam_slot, &mu_slot);
  const double kappa_u = (lam_slot + 5.0 / 6.0 * mu_slot) + 2.0 * (4.0 / 3.0 * mu_slot);
  const int nnz = (int)s->col_idx.size();
  Vec vals(nnz, 0.0);
  if (s->tri2d) {
    for (int e = 0; e < s->nt; ++e) {
      const int32_t* c = &s->cells[e * 3];
      const double* Xv[3] = {&s->X[c[0] * 3], &s->X[c[1] * 3], &s->X[c[2] * 3]};
      double M[9], L[9];
      element_mass_2d(Xv, s->rho, M);
      const double kappa =
          s->pd_diff_mode == 2 ? (s->lam(e) + 5.0 / 6.0 * s->mu(e)) + 2.0 * (4.0 / 3.0 * s->mu(e)) : kappa_u;
      element_laplace_2d(Xv, s->dt * s->dt * kappa, L);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          for (int a = 0; a < 3; ++a)
            vals[s->hess_dst[(size_t)e * 81 + (i * 3 + a) * 9 + j * 3 + a]] += M[i * 3 + j] + L[i * 3 + j];
    }
  } else
  for (int e = 0; e < s->nt; ++e) {
    const int32_t* c = &s->cells[e * 4];
    const double* Xv[4] = {&s->X[c[0] * 3], &s->X[c[1] * 3], &s->X[c[2] * 3], &s->X[c[3] * 3]};
    double M[16], L[16];
    element_mass(Xv, s->rho, M);
    const double kappa =
        s->pd_diff_mode == 2 ? (s->lam(e) + 5.0 / 6.0 * s->mu(e)) + 2.0 * (4.0 / 3.0 * s->mu(e)) : kappa_u;
    element_laplace(Xv, s->dt * s->dt * kappa, L);
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        for (int a = 0; a < 3; ++a)
          vals[s->hess_dst[(size_t)e * 144 + (i * 3 + a) * 12 + j * 3 + a]] += M[i * 4 + j] + L[i * 4 + j];
  }
  filter_dbc_matrix(*s, vals);
  s->pd_vals = vals;
  s->pd_ready = true;
  if (out) std::copy(vals.begin(), vals.end(), out);
}

double orc_compute_step_pd(orc_ts* s, const orc_params* p, orc_stats* st) {
  if (!s->pd_ready) orc_pd_matrix_values(s, nullptr);
  return lbfgs_core(s, p, st, 1);
}

// step_next (time_step.hpp:530-543)
void orc_step_next(orc_ts* s) {
  s->prev_deform = s->deformation;
  s->deformation = s->next;
  for (int i = 0; i < s->n; ++i)
    s->velocity[i] = (s->deformation[i] - s->prev_deform[i]) * (1.0 / s->dt) * (1 - s->damping);
}

// restore (time_step.hpp:560-569)
void orc_restore(orc_ts* s) {
  for (int i = 0; i < s->n; ++i)
    if (s->dbc(i)) {
      s->prev_deform[i] = s->dbc_values[i];
      s->deformation[i] = s->dbc_values[i];
    }
  for (int i = 0; i < s->n; ++i) s->velocity[i] = (s->deformation[i] - s->prev_deform[i]) * (1.0 / s->dt);
}

int orc_check_convergence(orc_ts* s) { return nrm2(s->forces) < s->abs_tol ? 1 : 0; }

static Vec* buf(orc_ts* s, int which) {
  switch (which) {
    case ORC_DEFORMATION: return &s->deformation;
    case ORC_PREV_DEFORM: return &s->prev_deform;
    case ORC_INERTIA_DEFORM: return &s->inertia;
    case ORC_NEXT_DEFORM: return &s->next;
    case ORC_VELOCITY: return &s->velocity;
    case ORC_EXT_ACCEL: return &s->ext_accel;
    case ORC_FORCES: return &s->forces;
    case ORC_DBC_VALUES: return &s->dbc_values;
  }
  return nullptr;
}
void orc_get(const orc_ts* s, int which, double* out) {
  const Vec* v = buf(const_cast<orc_ts*>(s), which);
  if (v) std::copy(v->begin(), v->end(), out);
}
void orc_set(orc_ts* s, int which, const double* in) {
  Vec* v = buf(s, which);
  if (v) std::copy(in, in + s->n, v->begin());
}
void orc_get_dminv(const orc_ts* s, double* out) { std::copy(s->dminv.begin(), s->dminv.end(), out); }
void orc_get_rest_vol(const orc_ts* s, double* out) { std::copy(s->vol.begin(), s->vol.end(), out); }
void orc_get_def_grad(const orc_ts* s, double* out) { std::copy(s->defgrad.begin(), s->defgrad.end(), out); }
void orc_get_local_stiffness(const orc_ts* s, double* out) { std::copy(s->local_K.begin(), s->local_K.end(), out); }
void orc_get_csr(const orc_ts* s, int32_t* rp, int32_t* ci) {
  std::copy(s->row_ptr.begin(), s->row_ptr.end(), rp);
  std::copy(s->col_idx.begin(), s->col_idx.end(), ci);
}
void orc_get_values(const orc_ts* s, int which, double* vals) {
  const Vec& v = which == ORC_SYSMATRIX ? s->sys_vals : (which == ORC_MASS ? s->mass_vals : s->massf_vals);
  std::copy(v.begin(), v.end(), vals);
}
void orc_spmv(const orc_ts* s, int which, const double* x, double* y) {
  const Vec& v = which == ORC_SYSMATRIX ? s->sys_vals : (which == ORC_MASS ? s->mass_vals : s->massf_vals);
  spmv(*s, v, x, y);
}
int orc_pcg(const orc_ts* s, const double* b, double* x, double rtol, int max_iters, int precond, double* rel_res) {
  return pcg(*s, s->sys_vals, b, x, rtol, max_iters, precond, rel_res);
}

// basic_gather_operator semantics with the composer's weights = rest volume (global_composer.hpp:36-128)
void orc_gather_force(const orc_ts* s, const double* lf, double alpha, double* f) {
  for (int v = 0; v < s->nv; ++v)
    for (int k = s->fcon_ptr[v]; k < s->fcon_ptr[v + 1]; ++k) {
      const int t = s->fcon_src[k];
      for (int d = 0; d < 3; ++d) f[v * 3 + d] += alpha * s->vol[t / 4] * lf[t * 3 + d];
    }
}
void orc_gather_hessian(const orc_ts* s, const double* K, double alpha, double* vals) {
  const int nnz = (int)s->col_idx.size();
  for (int k = 0; k < nnz; ++k)
    for (int q = s->hcon_ptr[k]; q < s->hcon_ptr[k + 1]; ++q) {
      const int t = s->hcon_src[q];
      vals[k] += alpha * s->vol[t / 144] * K[t];
    }
}

void orc_local_mass(const orc_ts* s, double alpha, double* out) {
  for (int e = 0; e < s->nt; ++e) {
    const int32_t* c = &s->cells[e * 4];
    const double* Xv[4] = {&s->X[c[0] * 3], &s->X[c[1] * 3], &s->X[c[2] * 3], &s->X[c[3] * 3]};
    element_mass(Xv, alpha, out + (size_t)e * 16);
  }
}
void orc_local_laplace(const orc_ts* s, double alpha, double* out) {
  for (int e = 0; e < s->nt; ++e) {
    const int32_t* c = &s->cells[e * 4];
    const double* Xv[4] = {&s->X[c[0] * 3], &s->X[c[1] * 3], &s->X[c[2] * 3], &s->X[c[3] * 3]};
    element_laplace(Xv, alpha, out + (size_t)e * 16);
  }
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
