// Host check of the strain-relative stable Neo-Hookean forms of elem_math.cuh (the FP32 element passes of
// the mixed path) against the direct formulas in FP64, over random materials and strains from 1e-4 to 3e-1:
// prints the worst errors of snh_eval_small (3D) and snh2_eval_small (2D) in FP64 and in FP32.
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
  return 0;
}
