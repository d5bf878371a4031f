// Calls the gravity model the way the patched TFM.cpp calls it: std::vector
// inputs shaped like FM::FM's (61x61x33 grid, fh = 1, fv = 2, bfr = 10, the
// node list nn of TFM.cpp:89), through ztm::gfm of include/ztm_grav.hpp on
// the GPU, and compares the field with the reference's own CPU lambda
// (TFM.cpp:95-99, compiled from TFM.cpp into oracle/_ref/libref_tfm.so).
// Exit status 0 when the double field agrees to 1e-12 (normwise relative)
// and the stations outside the bfr interior hold 0.
#include <math.h>
#include <stdio.h>

#include <vector>

#include "ztm_grav.hpp"

extern "C" void ref_tfm_gfm(int di, int dj, int dk, int fh, int fv, int bfr, const double* drho,
                            long long N, const int* nn, long long n_nn, const double* surf,
                            double* G);

int main() {
  const int di = 61, dj = 61, dk = 33, fh = 1, fv = 2, bfr = 10;
  const int ii = (di - 1) * fh + 1, jj = (dj - 1) * fh + 1, kk = (dk - 1) * fv + 1;
  const long long N = (long long)ii * jj * kk;
  // seeded inputs: a smooth density anomaly with a Moho-like step, stations
  // on a surface near the top of the grid (k up), nodes deeper than 1 unit
  unsigned long long st = 12345;
  auto rnd = [&]() {
    st = st * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(st >> 11) * (1.0 / 9007199254740992.0);
  };
  std::vector<double> drho(N, 0.0), surf(di * dj), G;
  std::vector<int> nn;
  for (int m = 0; m < di * dj; m++) surf[m] = (dk - 3) + 0.37 + 0.2 * rnd();
  for (long long n = 0; n < N; n++) {
    const double i = (double)(n % ii) / fh, j = (double)((n / ii) % jj) / fh,
                 k = (double)(n / ((long long)ii * jj)) / fv;
    double d = 0.3 * sin(i / 7.0) * cos(j / 5.0) * exp(-(k - 12.0) * (k - 12.0) / 40.0);
    d += (k < 10.0 + 2.0 * sin(i / 11.0)) ? -0.25 : 0.0;
    d += 0.02 * (rnd() - 0.5);
    if (k > (dk - 3) - 1.0) d = 0.0;
    if (fabs(d) > .001) {  // TFM.cpp:89
      drho[n] = d;
      nn.push_back((int)n);
    }
  }
  const int rc = ztm::gfm(drho, surf, G, nn, di, dj, dk, fh, fv, bfr);
  if (rc != 0) {
    fprintf(stderr, "ztm::gfm failed with status %d\n", rc);
    return 2;
  }
  std::vector<double> R(di * dj, 0.0);
  ref_tfm_gfm(di, dj, dk, fh, fv, bfr, drho.data(), N, nn.data(), (long long)nn.size(),
              surf.data(), R.data());
  double emax = 0.0, rmax = 0.0;
  int outside_nonzero = 0;
  for (int j0 = 0; j0 < dj; j0++)
    for (int i0 = 0; i0 < di; i0++) {
      const int m = i0 + j0 * di;
      const bool in = i0 >= bfr && i0 < di - bfr && j0 >= bfr && j0 < dj - bfr;
      if (!in) {
        if (G[m] != 0.0) outside_nonzero++;
        continue;
      }
      emax = fmax(emax, fabs(G[m] - R[m]));
      rmax = fmax(rmax, fabs(R[m]));
    }
  const double rel = emax / rmax;
  printf("nodes %zu  max|G| %.6g mGal  normwise rel err %.3e  nonzero outside interior %d\n",
         nn.size(), rmax, rel, outside_nonzero);
  return (rel <= 1e-12 && outside_nonzero == 0 && rmax > 0) ? 0 : 1;
}
