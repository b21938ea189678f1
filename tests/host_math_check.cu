// Host check of the strain-relative stable Neo-Hookean forms of elem_math.cuh (the FP32 element passes of
// the mixed path) against the direct formulas in FP64, over random materials and strains from 1e-4 to 3e-1:
// prints the worst errors of snh_eval_small (3D) and snh2_eval_small (2D) in FP64 and in FP32, and of the
// increment form snh_increment (3D) against the direct formulas' differences in long double.
// Built and run by tests/test_host_math.py with nvcc as host code.
#include <cmath>
#include <cstdio>
#include <random>

#include "elem_math.cuh"

using namespace ssim_gb;

namespace {

struct Worst {
  double e64 = 0, p64 = 0, e32 = 0, p32 = 0;
};

// direct 3D form: Psi = 1/2 [mu (Ic - 3) + lambda (J - alpha)^2 - mu log(Ic + 1)] - Psi(I),
// P = lambda (J - alpha) cof F + mu (1 - 1/(Ic + 1)) F, alpha = 1 + 3/4 mu / lambda
void check3(std::mt19937& rng, Worst& w) {
  std::uniform_real_distribution<double> U(-1, 1);
  const double lam = 1e4 * std::exp(4 * (U(rng) + 1)), mu = lam * (0.05 + 0.45 * (U(rng) + 1));
  const double alpha = 1 + 0.75 * mu / lam, psi0 = 0.5 * (lam * (1 - alpha) * (1 - alpha) - mu * std::log(4.0));
  const double amp = std::pow(10.0, -4 + 3.5 * (U(rng) + 1) / 2);
  double G[9], F[9];
  for (int k = 0; k < 9; ++k) {
    G[k] = amp * U(rng);
    F[k] = G[k] + (k % 4 == 0 ? 1 : 0);
  }
  double Ic = 0;
  for (int k = 0; k < 9; ++k) Ic += F[k] * F[k];
  const double J = det3(F);
  const double psi = 0.5 * (mu * (Ic - 3) + lam * (J - alpha) * (J - alpha) - mu * std::log(Ic + 1)) - psi0;
  double C[9];
  cofactor(F, C);
  double Pd[9], pn = 0;
  for (int k = 0; k < 9; ++k) {
    Pd[k] = lam * (J - alpha) * C[k] + mu * (1 - 1 / (Ic + 1)) * F[k];
    pn += Pd[k] * Pd[k];
  }
  double P[9], sc;
  const double e = snh_eval_small<double, true>(G, lam, mu, P, sc);
  float Gf[9], Pf[9], scf;
  for (int k = 0; k < 9; ++k) Gf[k] = (float)G[k];
  const float ef = snh_eval_small<float, true>(Gf, (float)lam, (float)mu, Pf, scf);
  double dp = 0, dpf = 0;
  for (int k = 0; k < 9; ++k) {
    dp += (P[k] - Pd[k]) * (P[k] - Pd[k]);
    dpf += (Pf[k] - P[k]) * (Pf[k] - P[k]);
  }
  w.e64 = std::fmax(w.e64, std::fabs(e - psi) / sc);
  w.p64 = std::fmax(w.p64, std::sqrt(dp) / (mu * amp + std::sqrt(pn)));
  w.e32 = std::fmax(w.e32, std::fabs(ef - e) / sc);
  w.p32 = std::fmax(w.p32, std::sqrt(dpf) / (mu * amp + std::sqrt(pn)));
}

// direct 2D form with delta the positive root of (2t + 1) d^2 + (2t + 2) d - 2t = 0, t = mu / lambda
void check2(std::mt19937& rng, Worst& w) {
  std::uniform_real_distribution<double> U(-1, 1);
  const double lam = 1e4 * std::exp(4 * (U(rng) + 1)), mu = lam * (0.05 + 0.45 * (U(rng) + 1));
  const double t = mu / lam, a = 2 * t + 1, b = 2 * t + 2, c = -2 * t;
  const double delta = (-b + std::sqrt(b * b - 4 * a * c)) / (2 * a);
  const double alpha = (1 - 1 / (2 + delta)) * mu / lam + 1;
  const double psi0 = 0.5 * (lam * (1 - alpha) * (1 - alpha) - mu * std::log(2 + delta));
  const double amp = std::pow(10.0, -4 + 3.5 * (U(rng) + 1) / 2);
  double G[4], F[4];
  for (int k = 0; k < 4; ++k) {
    G[k] = amp * U(rng);
    F[k] = G[k] + ((k == 0 || k == 3) ? 1 : 0);
  }
  const double Ic = F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3], J = F[0] * F[3] - F[1] * F[2];
  const double psi = 0.5 * (mu * (Ic - 2) + lam * (J - alpha) * (J - alpha) - mu * std::log(Ic + delta)) - psi0;
  const double cf[4] = {F[3], -F[2], -F[1], F[0]};
  double Pd[4], pn = 0;
  for (int k = 0; k < 4; ++k) {
    Pd[k] = lam * (J - alpha) * cf[k] + mu * (1 - 1 / (Ic + delta)) * F[k];
    pn += Pd[k] * Pd[k];
  }
  double P[4], sc;
  const double e = snh2_eval_small<double, true>(G, lam, mu, delta, P, sc);
  float Gf[4] = {(float)G[0], (float)G[1], (float)G[2], (float)G[3]}, Pf[4], scf;
  const float ef = snh2_eval_small<float, true>(Gf, (float)lam, (float)mu, (float)delta, Pf, scf);
  double dp = 0, dpf = 0;
  for (int k = 0; k < 4; ++k) {
    dp += (P[k] - Pd[k]) * (P[k] - Pd[k]);
    dpf += (Pf[k] - P[k]) * (Pf[k] - P[k]);
  }
  w.e64 = std::fmax(w.e64, std::fabs(e - psi) / sc);
  w.p64 = std::fmax(w.p64, std::sqrt(dp) / (mu * amp + std::sqrt(pn)));
  w.e32 = std::fmax(w.e32, std::fabs(ef - e) / sc);
  w.p32 = std::fmax(w.p32, std::sqrt(dpf) / (mu * amp + std::sqrt(pn)));
}

// increment form: Gr of amplitude 1e-4 .. 3e-1, dG of 1e-7 .. 1e-1 of that; the direct differences
// P(Gr + dG) - P(Gr) and Psi(Gr + dG) - Psi(Gr) in long double; errors relative to |dP| and to the
// increment's energy scale mu |Gr| |dG| + lambda |dJ|
struct WorstInc {
  double p64 = 0, e64 = 0, p32 = 0, e32 = 0;
};

template <typename R>
void direct_pe(const R* F, R lam, R mu, R* P, R& psi) {
  R Ic = 0;
  for (int k = 0; k < 9; ++k) Ic += F[k] * F[k];
  const R alpha = 1 + R(0.75) * mu / lam;
  const R C[9] = {F[4] * F[8] - F[5] * F[7], F[5] * F[6] - F[3] * F[8], F[3] * F[7] - F[4] * F[6],
                  F[7] * F[2] - F[8] * F[1], F[8] * F[0] - F[6] * F[2], F[6] * F[1] - F[7] * F[0],
                  F[1] * F[5] - F[2] * F[4], F[2] * F[3] - F[0] * F[5], F[0] * F[4] - F[1] * F[3]};
  const R J = F[0] * C[0] + F[1] * C[1] + F[2] * C[2];
  for (int k = 0; k < 9; ++k) P[k] = lam * (J - alpha) * C[k] + mu * (1 - 1 / (Ic + 1)) * F[k];
  psi = R(0.5) * (mu * (Ic - 3) + lam * (J - alpha) * (J - alpha) - mu * std::log(Ic + 1));
}

void check_increment(std::mt19937& rng, WorstInc& w) {
  std::uniform_real_distribution<double> U(-1, 1);
  const double lam = 1e4 * std::exp(4 * (U(rng) + 1)), mu = lam * (0.05 + 0.45 * (U(rng) + 1));
  const double amp = std::pow(10.0, -4 + 3.5 * (U(rng) + 1) / 2);
  const double damp = amp * std::pow(10.0, -7 + 6 * (U(rng) + 1) / 2);
  double Gr[9], dG[9];
  long double Fa[9], Fb[9];
  for (int k = 0; k < 9; ++k) {
    Gr[k] = amp * U(rng);
    dG[k] = damp * U(rng);
    Fa[k] = (long double)Gr[k] + (k % 4 == 0 ? 1 : 0);
    Fb[k] = Fa[k] + (long double)dG[k];
  }
  long double Pa[9], Pb[9], ea, eb;
  direct_pe<long double>(Fa, lam, mu, Pa, ea);
  direct_pe<long double>(Fb, lam, mu, Pb, eb);
  double dPr[9], n = 0, gn = 0, dn = 0;
  for (int k = 0; k < 9; ++k) {
    dPr[k] = (double)(Pb[k] - Pa[k]);
    n += dPr[k] * dPr[k];
    gn += Gr[k] * Gr[k];
    dn += dG[k] * dG[k];
  }
  const double de = (double)(eb - ea);
  const double escale = (mu + lam) * (1 + std::sqrt(gn)) * std::sqrt(dn);
  double dP[9];
  const double e = snh_increment<double>(Gr, dG, lam, mu, dP);
  float Grf[9], dGf[9], dPf[9];
  for (int k = 0; k < 9; ++k) {
    Grf[k] = (float)Gr[k];
    dGf[k] = (float)dG[k];
  }
  const float ef = snh_increment<float>(Grf, dGf, (float)lam, (float)mu, dPf);
  double e1 = 0, e2 = 0;
  for (int k = 0; k < 9; ++k) {
    e1 += (dP[k] - dPr[k]) * (dP[k] - dPr[k]);
    e2 += (dPf[k] - dPr[k]) * (dPf[k] - dPr[k]);
  }
  w.p64 = std::fmax(w.p64, std::sqrt(e1 / n));
  w.p32 = std::fmax(w.p32, std::sqrt(e2 / n));
  w.e64 = std::fmax(w.e64, std::fabs(e - de) / escale);
  w.e32 = std::fmax(w.e32, std::fabs(ef - de) / escale);
}

}  // namespace

int main() {
  std::mt19937 rng(7);
  Worst w3, w2;
  for (int i = 0; i < 4000; ++i) {
    check3(rng, w3);
    check2(rng, w2);
  }
  std::printf("3d %.3e %.3e %.3e %.3e\n", w3.e64, w3.p64, w3.e32, w3.p32);
  std::printf("2d %.3e %.3e %.3e %.3e\n", w2.e64, w2.p64, w2.e32, w2.p32);
  WorstInc wi;
  for (int i = 0; i < 4000; ++i) check_increment(rng, wi);
  std::printf("inc %.3e %.3e %.3e %.3e\n", wi.e64, wi.p64, wi.e32, wi.p32);
  return 0;
}
