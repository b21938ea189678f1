// elem_math.cuh -- per-tet math in registers: deformation gradient, stable Neo-Hookean energy / PK1,
// and the SPD-projected 12x12 element stiffness through the analytic eigensystem of the 9x9 Hessian.
//
// Conventions (identical to the reference's views): F is the row-major deformation gradient
// F(r, c) = sum_k Ds(r, k) Dminv(k, c) (def_grad.hpp:93-132); the 9x9 Hessian index is r*3 + c of F;
// the 12x12 stiffness index is vertex*3 + dof (compute_pfpx_3, internal_physic.hpp:107-160).
#pragma once
#include <cuda_runtime.h>

namespace ssim_gb {

template <typename S>
__host__ __device__ __forceinline__ S det3(const S* A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}

// dJ/dF: rows of cof(F) are cross products of rows of F (partial_determinant,
// internal_physic.hpp:41-48, applied to the transposed matrix the model receives)
template <typename S>
__host__ __device__ __forceinline__ void cofactor(const S* F, S* C) {
  C[0] = F[4] * F[8] - F[5] * F[7];
  C[1] = F[5] * F[6] - F[3] * F[8];
  C[2] = F[3] * F[7] - F[4] * F[6];
  C[3] = F[7] * F[2] - F[8] * F[1];
  C[4] = F[8] * F[0] - F[6] * F[2];
  C[5] = F[6] * F[1] - F[7] * F[0];
  C[6] = F[1] * F[5] - F[2] * F[4];
  C[7] = F[2] * F[3] - F[0] * F[5];
  C[8] = F[0] * F[4] - F[1] * F[3];
}

// stable Neo-Hookean, delta = 1 (stable_neohookean.hpp:23-62, 93-104):
//   Psi = 1/2 [mu (Ic - 3) + lambda (J - alpha)^2 - mu log(Ic + 1)] - Psi0,  alpha = 1 + 3/4 mu/lambda
//   P   = lambda (J - alpha) cof(F) + mu (1 - 1/(Ic + 1)) F
template <typename S>
__host__ __device__ __forceinline__ S snh_energy(const S* F, S lam, S mu) {
  S Ic = 0;
#pragma unroll
  for (int i = 0; i < 9; ++i) Ic += F[i] * F[i];
  const S alpha = S(0.75) * mu / lam + S(1);
  const S Jm = det3(F) - alpha;
  const S zero_energy = S(0.5) * (lam * (S(1) - alpha) * (S(1) - alpha) - mu * log(S(4)));
  return S(0.5) * (mu * (Ic - S(3)) + lam * Jm * Jm - mu * log(Ic + S(1))) - zero_energy;
}

template <typename S>
__host__ __device__ __forceinline__ S snh_stress(const S* F, S lam, S mu, S* P) {
  S Ic = 0;
#pragma unroll
  for (int i = 0; i < 9; ++i) Ic += F[i] * F[i];
  const S alpha = S(0.75) * mu / lam + S(1);
  const S Jm = det3(F) - alpha;
  S C[9];
  cofactor(F, C);
  const S s = mu * (S(1) - S(1) / (Ic + S(1)));
  const S lj = lam * Jm;
#pragma unroll
  for (int i = 0; i < 9; ++i) P[i] = lj * C[i] + s * F[i];
  const S zero_energy = S(0.5) * (lam * (S(1) - alpha) * (S(1) - alpha) - mu * log(S(4)));
  return S(0.5) * (mu * (Ic - S(3)) + lam * Jm * Jm - mu * log(Ic + S(1))) - zero_energy;
}

// Energy, first Piola-Kirchhoff stress (when STRESS) and the sum of the magnitudes of the energy's terms
// in one pass sharing I_c, J and log(I_c + 1); alpha = 1 + 3/4 mu / lambda and psi0 = the energy's value
// at F = I (stable_neohookean.hpp:34,60) come precomputed per element.  Same formulas as snh_stress /
// snh_energy / snh_energy_scale.
template <typename S, bool STRESS>
__host__ __device__ __forceinline__ S snh_eval(const S* F, S lam, S mu, S alpha, S psi0, S* P, S& scale) {
  S Ic = 0;
#pragma unroll
  for (int i = 0; i < 9; ++i) Ic += F[i] * F[i];
  S C[9];
  S J;
  if (STRESS) {
    cofactor(F, C);
    J = F[0] * C[0] + F[1] * C[1] + F[2] * C[2];
  } else {
    J = det3(F);
  }
  const S Jm = J - alpha;
  if (STRESS) {
    const S sF = mu * (S(1) - S(1) / (Ic + S(1)));
    const S lj = lam * Jm;
#pragma unroll
    for (int i = 0; i < 9; ++i) P[i] = lj * C[i] + sF * F[i];
  }
  const S t1 = mu * (Ic - S(3)), t2 = lam * Jm * Jm, t3 = mu * log(Ic + S(1));
  scale = S(0.5) * (fabs(t1) + t2 + fabs(t3)) + fabs(psi0);
  return S(0.5) * (t1 + t2 - t3) - psi0;
}

// cof(A + B) - cof(A) - cof(B): the part of the cofactor (quadratic in its argument) bilinear in A and B,
// for cofactor()'s convention C[k] = F[a] F[b] - F[c] F[d]
template <typename S>
__host__ __device__ __forceinline__ void cofactor_cross(const S* A, const S* B, S* C) {
  constexpr int idx[9][4] = {{4, 8, 5, 7}, {5, 6, 3, 8}, {3, 7, 4, 6}, {7, 2, 8, 1}, {8, 0, 6, 2},
                             {6, 1, 7, 0}, {1, 5, 2, 4}, {2, 3, 0, 5}, {0, 4, 1, 3}};
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int a = idx[k][0], b = idx[k][1], c = idx[k][2], d = idx[k][3];
    C[k] = A[a] * B[b] + B[a] * A[b] - A[c] * B[d] - B[c] * A[d];
  }
}

// The stable Neo-Hookean energy and PK1 increments between the displacement gradients Gr and Gr + dG,
// written so that each term is proportional to dG (rounding relative to the increment, not to the stress):
// with F = Fr + dG, s = Ic - 3, a(s) = 1 - 1/(s + 4), c1 = -3/4 mu / lambda,
//   ds   = 2 Fr:dG + |dG|^2
//   dJ   = cof(Fr):dG + Fr:cof(dG) + det(dG)                       (det of a sum of 3x3 matrices)
//   dcof = cross(Fr, dG) + cof(dG)
//   da   = ds / ((sr + 4)(sr + ds + 4))
//   dP   = lambda [(Jr - alpha) dcof + dJ (cof Fr + dcof)] + mu [a(sr) dG + da (Fr + dG)]
//   dPsi = 1/2 [ mu (ds - log1p(ds / (sr + 4))) + lambda dJ ((J - 1) + (Jr - 1) + 2 c1) ]
// (the differences of snh_eval_small's energy and stress, expanded exactly).  The reference quantities
// (Fr, cof Fr, sr, Jr - 1) only scale the increment's terms, so their own rounding perturbs the result
// relative to the increment too.
template <typename S>
__host__ __device__ __forceinline__ S snh_increment(const S* Gr, const S* dG, S lam, S mu, S* dP) {
  S Fr[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Fr[k] = Gr[k] + (k % 4 == 0 ? S(1) : S(0));
  // reference: sr = 2 tr Gr + |Gr|^2, Jr - 1 from the principal minors of Gr (as snh_eval_small)
  const S trGr = Gr[0] + Gr[4] + Gr[8];
  S n2 = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) n2 += Gr[k] * Gr[k];
  const S sr = S(2) * trGr + n2;
  S cGr[9];
  cofactor(Gr, cGr);
  const S Jr1 = trGr + (cGr[0] + cGr[4] + cGr[8]) + (Gr[0] * cGr[0] + Gr[1] * cGr[1] + Gr[2] * cGr[2]);
  S cFr[9];
  cofactor(Fr, cFr);
  // increments
  S fd = 0, d2 = 0, cd = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    fd += Fr[k] * dG[k];
    d2 += dG[k] * dG[k];
    cd += cFr[k] * dG[k];
  }
  const S ds = S(2) * fd + d2;
  S cdG[9], dC[9];
  cofactor(dG, cdG);
  cofactor_cross(Fr, dG, dC);
  S fc = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    fc += Fr[k] * cdG[k];
    dC[k] += cdG[k];
  }
  const S detdG = dG[0] * cdG[0] + dG[1] * cdG[1] + dG[2] * cdG[2];
  const S dJ = cd + fc + detdG;
  const S c1 = S(-0.75) * mu / lam;
  const S Jm_r = Jr1 + c1;  // Jr - alpha
  const S ar = (sr + S(3)) / (sr + S(4));
  const S da = ds / ((sr + S(4)) * (sr + ds + S(4)));
  if (dP != nullptr) {
#pragma unroll
    for (int k = 0; k < 9; ++k)
      dP[k] = lam * (Jm_r * dC[k] + dJ * (cFr[k] + dC[k])) + mu * (ar * dG[k] + da * (Fr[k] + dG[k]));
  }
  const S dlog = log1p(ds / (sr + S(4)));
  return S(0.5) * (mu * (ds - dlog) + lam * dJ * ((Jr1 + dJ) + Jr1 + S(2) * c1));
}

// The stable Neo-Hookean energy and PK1 written in the displacement gradient G = F - I so that no O(mu) or
// O(lambda) terms cancel (for FP32 evaluation of small strains): with s = Ic - 3 = 2 tr G + |G|^2,
// J - 1 = tr G + (principal 2x2 minors of G) + det G, c1 = 1 - alpha = -3/4 mu / lambda:
//   Psi - Psi(I) = 1/2 [ mu (s - log1p(s / 4)) + lambda (J - 1)(J - 1 + 2 c1) ]
//   P = lambda (J - 1) cof F + 3/4 mu (G + G^T - tr G I - cof G) + mu s / (4 (4 + s)) F,
// using cof(I + G) = I + tr G I - G^T + cof G.  Algebraically the same functions as snh_eval (the
// reference's stable_neohookean.hpp:23-62); scale returns the magnitude sum of the terms above.
template <typename S, bool STRESS>
__host__ __device__ __forceinline__ S snh_eval_small(const S* G, S lam, S mu, S* P, S& scale) {
  const S trG = G[0] + G[4] + G[8];
  S n2 = 0;
#pragma unroll
  for (int i = 0; i < 9; ++i) n2 += G[i] * G[i];
  const S s = S(2) * trG + n2;
  S cG[9];
  cofactor(G, cG);
  const S m2 = cG[0] + cG[4] + cG[8];  // sum of the principal 2x2 minors
  const S dG = G[0] * cG[0] + G[1] * cG[1] + G[2] * cG[2];
  const S Jm1 = trG + m2 + dG;
  const S c1 = S(-0.75) * mu / lam;
  const S lg = log1p(S(0.25) * s);
  if (STRESS) {
    const S lj = lam * Jm1, q = mu * s / (S(4) * (S(4) + s)), h = S(0.75) * mu;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int k = r * 3 + c;
        const S id = r == c ? S(1) : S(0);
        const S cofF = id + (r == c ? trG : S(0)) - G[c * 3 + r] + cG[k];
        const S D = G[k] + G[c * 3 + r] - (r == c ? trG : S(0)) - cG[k];
        P[k] = lj * cofF + h * D + q * (id + G[k]);
      }
  }
  const S t1 = mu * (s - lg), t2 = lam * Jm1 * (Jm1 + S(2) * c1);
  scale = S(0.5) * (mu * (fabs(s) + fabs(lg)) + lam * fabs(Jm1) * (fabs(Jm1) + S(2) * fabs(c1)));
  return S(0.5) * (t1 + t2);
}

// The 2D stable Neo-Hookean (stable_neohookean.hpp with Ndim 2: Psi = 1/2 [mu (Ic - 2) + lambda (J - alpha)^2
// - mu log(Ic + delta)] - Psi(I), alpha = 1 + (1 - 1/(2 + delta)) mu / lambda) in the displacement gradient
// G = F - I (row-major 2x2), for FP32 evaluation of small strains: with s = Ic - 2 = 2 tr G + |G|^2,
// J - 1 = tr G + det G, h = (1 - 1/(2 + delta)) mu = lambda (alpha - 1) and C = cof G = [[G11, -G10],
// [-G01, G00]] (so cof F = I + C):
//   Psi - Psi(I) = 1/2 [ mu (s - log1p(s / (2 + delta))) + lambda (J - 1)(J - 1) - 2 h (J - 1) ]
//   P = lambda (J - 1)(I + C) + h (G - C) + mu s / ((2 + delta)(2 + delta + s)) (I + G),
// the expansion of P = lambda (J - alpha) cof F + mu (1 - 1/(Ic + delta)) F in which the rest terms
// (lambda (1 - alpha) + h = 0) cancel analytically; scale returns the magnitude sum of the terms.
template <typename S, bool STRESS>
__host__ __device__ __forceinline__ S snh2_eval_small(const S* G, S lam, S mu, S delta, S* P, S& scale) {
  const S trG = G[0] + G[3];
  const S s = S(2) * trG + (G[0] * G[0] + G[1] * G[1] + G[2] * G[2] + G[3] * G[3]);
  const S Jm1 = trG + (G[0] * G[3] - G[1] * G[2]);
  const S b = S(2) + delta;
  const S h = (S(1) - S(1) / b) * mu;
  const S lg = log1p(s / b);
  if (STRESS) {
    const S C[4] = {G[3], -G[2], -G[1], G[0]};
    const S lj = lam * Jm1, q = mu * s / (b * (b + s));
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const S id = (k == 0 || k == 3) ? S(1) : S(0);
      P[k] = lj * (id + C[k]) + h * (G[k] - C[k]) + q * (id + G[k]);
    }
  }
  const S t1 = mu * (s - lg), t2 = lam * Jm1 * Jm1 - S(2) * h * Jm1;
  scale = S(0.5) * (mu * (fabs(s) + fabs(lg)) + lam * Jm1 * Jm1 + S(2) * h * fabs(Jm1));
  return S(0.5) * (t1 + t2);
}

// per-element constants of snh_eval
template <typename S>
__host__ __device__ __forceinline__ void snh_constants(S lam, S mu, S& alpha, S& psi0) {
  alpha = S(0.75) * mu / lam + S(1);
  psi0 = S(0.5) * (lam * (S(1) - alpha) * (S(1) - alpha) - mu * log(S(4)));
}

// Linear elasticity (linear.hpp:23-68) from the displacement gradient G = F - I: eps = (G + G^T) / 2
// (approx_green_strain, internal_physic.hpp:27-30, without the cancellation of F + F^T - 2I),
// Psi = mu |eps|^2 + lambda/2 tr(eps)^2, P = 2 mu eps + lambda tr(eps) I.  Every term is non-negative, so
// the magnitude sum used for the line search's round-off slack is Psi itself.
template <typename S, bool STRESS>
__host__ __device__ __forceinline__ S linear_eval(const S* G, S lam, S mu, S* P, S& scale) {
  S e[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) e[r * 3 + c] = S(0.5) * (G[r * 3 + c] + G[c * 3 + r]);
  const S tr = e[0] + e[4] + e[8];
  S n2 = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) n2 += e[k] * e[k];
  if (STRESS) {
#pragma unroll
    for (int k = 0; k < 9; ++k) P[k] = S(2) * mu * e[k] + ((k % 4 == 0) ? lam * tr : S(0));
  }
  const S psi = mu * n2 + S(0.5) * lam * tr * tr;
  scale = psi;
  return psi;
}

// sum of the magnitudes of the terms of snh_energy: the scale of its absolute round-off (the terms are
// O(mu) and cancel to O(mu strain^2) near rest); the line search compares energies only above it
template <typename S>
__host__ __device__ __forceinline__ S snh_energy_scale(const S* F, S lam, S mu) {
  S Ic = 0;
#pragma unroll
  for (int i = 0; i < 9; ++i) Ic += F[i] * F[i];
  const S alpha = S(0.75) * mu / lam + S(1);
  const S Jm = det3(F) - alpha;
  const S zero_energy = S(0.5) * (lam * (S(1) - alpha) * (S(1) - alpha) - mu * log(S(4)));
  return S(0.5) * (mu * fabs(Ic - S(3)) + lam * Jm * Jm + mu * fabs(log(Ic + S(1)))) + fabs(zero_energy);
}

// ------------------------------------------------------------------ symmetric 3x3 eigen (cyclic Jacobi)
// A (row-major, symmetric) is diagonalised in place; Q accumulates the rotations (eigenvectors as
// columns).  Rotation of Golub & Van Loan Alg. 8.5.1 / Numerical Recipes 11.1.
template <typename S>
__host__ __device__ __forceinline__ void jacobi_rot(S* A, S* Q, int p, int q, int r) {
  const S apq = A[p * 3 + q];
  if (apq == S(0)) return;
  const S tau = (A[q * 3 + q] - A[p * 3 + p]) / (S(2) * apq);
  const S t = (tau >= S(0) ? S(1) : S(-1)) / (fabs(tau) + sqrt(S(1) + tau * tau));
  const S c = S(1) / sqrt(S(1) + t * t), s = t * c;
  A[p * 3 + p] -= t * apq;
  A[q * 3 + q] += t * apq;
  A[p * 3 + q] = A[q * 3 + p] = S(0);
  const S arp = A[r * 3 + p], arq = A[r * 3 + q];
  A[r * 3 + p] = A[p * 3 + r] = c * arp - s * arq;
  A[r * 3 + q] = A[q * 3 + r] = s * arp + c * arq;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const S qkp = Q[k * 3 + p], qkq = Q[k * 3 + q];
    Q[k * 3 + p] = c * qkp - s * qkq;
    Q[k * 3 + q] = s * qkp + c * qkq;
  }
}

template <typename S>
__host__ __device__ __forceinline__ void sym_eig3(S* A, S* Q) {
#pragma unroll
  for (int i = 0; i < 9; ++i) Q[i] = (i % 4 == 0) ? S(1) : S(0);
  const S eps = sizeof(S) == 8 ? S(1e-32) : S(1e-14);  // squared relative off-diagonal target
  for (int sweep = 0; sweep < 12; ++sweep) {
    const S off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
    const S dia = A[0] * A[0] + A[4] * A[4] + A[8] * A[8];
    if (!(off > eps * dia)) break;
    jacobi_rot(A, Q, 0, 1, 2);
    jacobi_rot(A, Q, 0, 2, 1);
    jacobi_rot(A, Q, 1, 2, 0);
  }
}

// Givens rotation on rows (i, j) zeroing B(j, c); U accumulates the transposes (B = U R).
template <typename S>
__host__ __device__ __forceinline__ void givens_qr(S* B, S* U, int i, int j, int c) {
  const S a = B[i * 3 + c], b = B[j * 3 + c];
  const S r = sqrt(a * a + b * b);
  S cs = S(1), sn = S(0);
  if (r > S(0)) {
    cs = a / r;
    sn = b / r;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const S bi = B[i * 3 + k], bj = B[j * 3 + k];
    B[i * 3 + k] = cs * bi + sn * bj;
    B[j * 3 + k] = -sn * bi + cs * bj;
    const S ui = U[k * 3 + i], uj = U[k * 3 + j];
    U[k * 3 + i] = cs * ui + sn * uj;
    U[k * 3 + j] = -sn * ui + cs * uj;
  }
}

template <typename S>
__host__ __device__ __forceinline__ void swap_cols_keep_det(S* V, S* d, int i, int j) {
  const S t = d[i];
  d[i] = d[j];
  d[j] = t;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const S a = V[k * 3 + i];
    V[k * 3 + i] = V[k * 3 + j];
    V[k * 3 + j] = -a;
  }
}

// Rotation-variant SVD F = U diag(s) V^T with U, V in SO(3), s0 >= s1 >= |s2|, s2 < 0 for inverted F.
// V from the Jacobi eigenvectors of F^T F, U and s from a Givens QR of F V (the approach of McAdams et
// al., "Computing the SVD of 3x3 matrices with minimal branching", 2011, written here with exact
// Jacobi rotations).
template <typename S>
__host__ __device__ __forceinline__ void svd3(const S* F, S* U, S* s, S* V) {
  S A[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) A[i * 3 + j] = F[0 * 3 + i] * F[0 * 3 + j] + F[1 * 3 + i] * F[1 * 3 + j] + F[2 * 3 + i] * F[2 * 3 + j];
  sym_eig3(A, V);
  S d[3] = {A[0], A[4], A[8]};
  if (d[0] < d[1]) swap_cols_keep_det(V, d, 0, 1);
  if (d[0] < d[2]) swap_cols_keep_det(V, d, 0, 2);
  if (d[1] < d[2]) swap_cols_keep_det(V, d, 1, 2);
  S B[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) B[i * 3 + j] = F[i * 3 + 0] * V[0 * 3 + j] + F[i * 3 + 1] * V[1 * 3 + j] + F[i * 3 + 2] * V[2 * 3 + j];
#pragma unroll
  for (int i = 0; i < 9; ++i) U[i] = (i % 4 == 0) ? S(1) : S(0);
  givens_qr(B, U, 0, 1, 0);
  givens_qr(B, U, 0, 2, 0);
  givens_qr(B, U, 1, 2, 1);
  s[0] = B[0];
  s[1] = B[4];
  s[2] = B[8];
}

// packed upper-triangular index of the 12x12 stiffness
__host__ __device__ constexpr int kup(int i, int j) { return i * 12 - (i * (i - 1)) / 2 + (j - i); }

template <typename S>
__host__ __device__ __forceinline__ void rank1(S* K, S w, const S* g) {
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    const S wi = w * g[i];
#pragma unroll
    for (int j = i; j < 12; ++j) K[kup(i, j)] += wi * g[j];
  }
}

// Element stiffness of the linear model, packed upper triangle (78) times scale.  Its 9x9 Hessian
// mu (I + T) + lambda d d^T (T: the transpose permutation, d = vec I) has the eigenspaces symmetric-
// deviatoric (2 mu, 5 modes), volumetric (2 mu + 3 lambda) and skew (0, 3 modes); with the make_spsd clamp
// (time_step.hpp:50-56) applied to those eigenvalues, H = c_I I + c_T T + c_d d d^T with
// c_I = (a_dev + a_skew)/2, c_T = (a_dev - a_skew)/2, c_d = (a_vol - a_dev)/3, and contracted with the shape
// gradients g_v: K[(v,s),(w,t)] = c_I delta_st g_v.g_w + c_T g_v[t] g_w[s] + c_d g_v[s] g_w[t].
template <typename S>
__host__ __device__ __forceinline__ void linear_stiffness(const S D[4][3], S lam, S mu, bool spsd, S scale, S* K) {
  S a_dev = S(2) * mu, a_vol = S(2) * mu + S(3) * lam, a_skew = S(0);
  if (spsd) {
    const S eps = S(1e-3);
    a_dev = fmax(a_dev, eps);
    a_vol = fmax(a_vol, eps);
    a_skew = eps;
  }
  const S cI = S(0.5) * (a_dev + a_skew) * scale, cT = S(0.5) * (a_dev - a_skew) * scale,
          cd = (a_vol - a_dev) / S(3) * scale;
#pragma unroll
  for (int v = 0; v < 4; ++v)
#pragma unroll
    for (int w = v; w < 4; ++w) {
      const S gg = D[v][0] * D[w][0] + D[v][1] * D[w][1] + D[v][2] * D[w][2];
#pragma unroll
      for (int s = 0; s < 3; ++s)
#pragma unroll
        for (int t = 0; t < 3; ++t) {
          const int i = v * 3 + s, j = w * 3 + t;
          if (i > j) continue;
          K[kup(i, j)] = (s == t ? cI * gg : S(0)) + cT * D[v][t] * D[w][s] + cd * D[v][s] * D[w][t];
        }
    }
}

// 12x12 element stiffness K = pfpx^T H+ pfpx (time_step.hpp:23-60) where H is the 9x9 SNH Hessian
// (stable_neohookean.hpp:64-91) and H+ = sum_m max(l_m, eps) e_m e_m^T (eps = 1e-3 absolute,
// time_step.hpp:52) when spsd, else H itself.  The eigensystem is analytic: with F = U S V^T,
//   a = mu (1 - 1/(I2 + 1)),  b = 2 mu / (I2 + 1)^2,  c = lambda (I3 - alpha)
// the six off-diagonal modes U (e_i e_j^T -+ e_j e_i^T) V^T / sqrt2 have eigenvalues a +- c s_k
// (k the third index), and the three scaling modes U diag(q) V^T come from the 3x3 block
//   A3 = a I + b s s^T + lambda g g^T + c [[0,s2,s1],[s2,0,s0],[s1,s0,0]],  g = (s1 s2, s0 s2, s0 s1)
// (the mode structure of Smith, de Goes & Kim, "Analytic Eigensystems for Isotropic Distortion
// Energies", 2019, derived here for this energy's I2/I3 form).  Each mode contracts with the shape
// gradients D (4x3) into a 12-vector G(v*3+a) = (E D^T)(a, v), and K accumulates l_m G G^T.
// Output: packed upper triangle (78 entries), times `scale`.
template <typename S>
__host__ __device__ __forceinline__ void element_stiffness(const S* F, const S D[4][3], S lam, S mu, bool spsd, S scale,
                                                  S* K) {
  S U[9], s[3], V[9];
  svd3(F, U, s, V);
  const S I2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
  const S I3 = s[0] * s[1] * s[2];
  const S alpha = S(0.75) * mu / lam + S(1);
  const S a = mu * (S(1) - S(1) / (I2 + S(1)));
  const S b = mu * (S(2) / ((I2 + S(1)) * (I2 + S(1))));
  const S c = lam * (I3 - alpha);
  const S eps = S(1e-3);
  // W = D V : W[v][j] = sum_l D[v][l] V[l][j]
  S W[4][3];
#pragma unroll
  for (int v = 0; v < 4; ++v)
#pragma unroll
    for (int j = 0; j < 3; ++j) W[v][j] = D[v][0] * V[0 * 3 + j] + D[v][1] * V[1 * 3 + j] + D[v][2] * V[2 * 3 + j];
#pragma unroll
  for (int i = 0; i < 78; ++i) K[i] = S(0);
  // twist / flip pairs (i, j) with remaining index k
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const int i = (m == 0) ? 1 : 0;
    const int j = (m == 2) ? 1 : 2;
    const int k = m;
    S lt = a + c * s[k];
    S lf = a - c * s[k];
    if (spsd) {
      lt = fmax(lt, eps);
      lf = fmax(lf, eps);
    }
    S gt[12], gf[12];
#pragma unroll
    for (int v = 0; v < 4; ++v)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const S x = U[d * 3 + i] * W[v][j];
        const S y = U[d * 3 + j] * W[v][i];
        gt[v * 3 + d] = x - y;
        gf[v * 3 + d] = x + y;
      }
    rank1(K, S(0.5) * lt * scale, gt);
    rank1(K, S(0.5) * lf * scale, gf);
  }
  // scaling block
  S A3[9], Q[9];
  const S g0 = s[1] * s[2], g1 = s[0] * s[2], g2 = s[0] * s[1];
  A3[0] = a + b * s[0] * s[0] + lam * g0 * g0;
  A3[4] = a + b * s[1] * s[1] + lam * g1 * g1;
  A3[8] = a + b * s[2] * s[2] + lam * g2 * g2;
  A3[1] = A3[3] = b * s[0] * s[1] + lam * g0 * g1 + c * s[2];
  A3[2] = A3[6] = b * s[0] * s[2] + lam * g0 * g2 + c * s[1];
  A3[5] = A3[7] = b * s[1] * s[2] + lam * g1 * g2 + c * s[0];
  sym_eig3(A3, Q);
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    S l = A3[m * 4];
    if (spsd) l = fmax(l, eps);
    S g[12];
#pragma unroll
    for (int v = 0; v < 4; ++v)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        g[v * 3 + d] = Q[0 * 3 + m] * U[d * 3 + 0] * W[v][0] + Q[1 * 3 + m] * U[d * 3 + 1] * W[v][1] +
                       Q[2 * 3 + m] * U[d * 3 + 2] * W[v][2];
    rank1(K, l * scale, g);
  }
}

}  // namespace ssim_gb
