// host_igk.cpp -- k+G sphere ordering of Quantum ESPRESSO (host code).
//
// Restates gk_sort and hpsort_eps of Modules/qe_gksort.f90:44-203 (adapted
// there from QE 6.5 PW/src/gk_sort.f90 and Modules/sort.f90): the k+G vectors
// with |k+G|^2 <= ecut, heap-sorted by |k+G|^2 with values closer than 1e-8
// ordered by G index.  The ordering defines which coefficient belongs to which
// G vector, so it is reproduced operation by operation.
#include <cmath>

namespace rpa {

static void hpsort_eps(int n, double* ra0, int* ind0, double eps) {
  double* ra = ra0 - 1;
  int* ind = ind0 - 1;
  if (n >= 1 && ind[1] == 0)
    for (int i = 1; i <= n; ++i) ind[i] = i;
  if (n < 2) return;
  int l = n / 2 + 1, ir = n;
  for (;;) {
    double rra;
    int iind;
    if (l > 1) {
      --l;
      rra = ra[l];
      iind = ind[l];
    } else {
      rra = ra[ir];
      iind = ind[ir];
      ra[ir] = ra[1];
      ind[ir] = ind[1];
      if (--ir == 1) {
        ra[1] = rra;
        ind[1] = iind;
        return;
      }
    }
    int i = l, j = l + l;
    while (j <= ir) {
      if (j < ir) {
        if (std::fabs(ra[j] - ra[j + 1]) >= eps) {
          if (ra[j] < ra[j + 1]) ++j;
        } else if (ind[j] < ind[j + 1]) {
          ++j;
        }
      }
      bool demote;
      if (std::fabs(rra - ra[j]) >= eps) demote = rra < ra[j];
      else demote = iind < ind[j];
      if (demote) {
        ra[i] = ra[j];
        ind[i] = ind[j];
        i = j;
        j += j;
      } else {
        j = ir + 1;
      }
    }
    ra[i] = rra;
    ind[i] = iind;
  }
}

int gk_sort_host(const double* k, int npwx, int ngm, const double* g, double ecut, int* ngk_out, int* igk,
                 double* gk) {
  const double eps8 = 1.0e-8;
  double q2x = std::sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]) + std::sqrt(ecut);
  q2x = q2x * q2x;
  for (int i = 0; i < npwx; ++i) {
    igk[i] = 0;
    gk[i] = 0.0;
  }
  int ngk = 0;
  bool stopped = false;
  for (int ng = 1; ng <= ngm; ++ng) {
    const double* gg = g + 3 * (ng - 1);
    double a = k[0] + gg[0], b = k[1] + gg[1], c = k[2] + gg[2];
    double q = a * a + b * b + c * c;
    if (q <= eps8) q = 0.0;
    if (q <= ecut) {
      if (++ngk > npwx) return -1;
      gk[ngk - 1] = q;
      igk[ngk - 1] = ng;
    } else if (gg[0] * gg[0] + gg[1] * gg[1] + gg[2] * gg[2] > q2x + eps8) {
      stopped = true;
      break;
    }
  }
  if (!stopped) return -2;
  hpsort_eps(ngk, gk, igk, eps8);
  for (int nk = 0; nk < ngk; ++nk) {
    const double* gg = g + 3 * (igk[nk] - 1);
    double a = k[0] + gg[0], b = k[1] + gg[1], c = k[2] + gg[2];
    gk[nk] = a * a + b * b + c * c;
  }
  *ngk_out = ngk;
  return 0;
}

}  // namespace rpa
