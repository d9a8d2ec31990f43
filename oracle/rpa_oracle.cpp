// rpa_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU FP64 restatement of the RPA response hot path of 2DMaterialsOpticalProps
// (Chi_RPA/Optabs.f90, W/Sloss.f90, W/gjel.f, Modules/qe_gksort.f90,
// Modules/vertices.f90).  It is the checker for the CUDA library and the timed
// CPU baseline; nothing in the product links, loads or calls it.
//
// The loops keep the reference's decomposition on purpose: an OpenMP `for`
// over FBZ k-points, a per-k private partial of S0 that is zeroed per k and
// added into the shared S0 inside a critical section (Sloss.f90:309-438,
// Optabs.f90:291-471), the Gfast index map built by a float-eps linear search
// at the first band pair of each k (Sloss.f90:905-944), per-element KK sums
// (Sloss.f90:954-1059, Optabs.f90:1112-1318), Gauss-Jordan with full pivoting
// (W/gjel.f:1-91) and the 4-deep W loop (Sloss.f90:1255-1277).
//
// Parity status: the reference ships no golden vectors and its Fortran does
// not build in this image (no Fortran compiler, iotk and MKL absent), so this
// restatement is pinned by analytic known-answer tests and by an independent
// numpy restatement (oracle/np_oracle.py), not by reference outputs.
//
// Array conventions follow the Fortran column-major layouts of the drivers;
// all indices handed in (K1, R1, K2, R2, iG0, igk) are 1-based as in Fortran.

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

typedef std::complex<double> cplx;

extern "C" {

// Pol codes shared with the product library (include/rpa_gpu.h).
enum { ORC_POL_XX = 0, ORC_POL_YY = 1, ORC_POL_ZZ = 2, ORC_POL_YZ = 3, ORC_POL_ZY = 4 };

struct OrcSystem {
  int ng;               // NG: number of G vectors
  const double* G;      // G(3,NG), Cartesian, 2pi/a0 units
  int nks, nbnd, npwx;  // IBZ k-points, bands, leading dim of coefficient blocks
  const int* npw;       // npw(nks): igwx of each IBZ k-point
  const int* igk;       // igk_k(npwx,nks), 1-based into G; NULL => coefficient i <-> G(:,i)
  const double* coeff;  // complex (re,im) C(npwx,nbnd,nks)
  const double* E;      // E(nks,nbnd), Hartree
  const double* R;      // R(48,3,3) Cartesian point-group operations
  const double* RI;     // RI(48,3,3) inverses
  int ntot;             // FBZ k-points
  const double* ktot;   // ktot(3,ntot), 2pi/a0 units
  const int* K1;        // K = R1*K1
  const int* R1;
  const int* K2;        // K+Q = G0 + R2*K2
  const int* R2;
  const int* iG0;
  int nlf;              // local fields
  const double* Glf;    // Glf(3,nlf), 2pi/a0 units
  double q[3];          // q, 2pi/a0 units
};

struct OrcParams {
  int ngd;       // legacy coefficient count NGd (ignored when igk != NULL)
  int nocc;      // Sloss: occupied bands (n <= nocc < m)
  int no;        // frequencies
  int pol;       // Optabs polarisation
  int nthreads;  // OpenMP threads
  int nk_list;   // >0: only process the FBZ k-points in klist (0-based)
  const int* klist;
  double domega, eta, T, Efermi, lor_cut, df_cut, Vcell, Gcar, eps;
};

// ---------------------------------------------------------------------------
// a5: Fermi-Dirac occupation, Optabs.f90:935-951.
void orc_occupation(double Ei, double Ef, double T, double* expo, double* f) {
  double x = (Ei - Ef) / T;
  if (x < -20) {
    *expo = 0.0;
    *f = 1.0;
  } else if (x > 20) {
    *expo = x;
    *f = 0.0;
  } else {
    *expo = std::exp(x);
    *f = 1.0 / (*expo + 1.0);
  }
}

// ---------------------------------------------------------------------------
// a1: heapsort with eps ties, Modules/qe_gksort.f90:96-203 (QE 6.5 sort.f90).
// ra, ind are 1-based arrays passed as 0-based pointers of length n.
void orc_hpsort_eps(int n, double* ra0, int* ind0, double eps) {
  double* ra = ra0 - 1;  // 1-based views
  int* ind = ind0 - 1;
  if (n >= 1 && ind[1] == 0) {
    for (int i = 1; i <= n; ++i) ind[i] = i;
  }
  if (n < 2) return;
  int l = n / 2 + 1, ir = n, i, j, iind;
  double rra;
  for (;;) {
    if (l > 1) {
      l = l - 1;
      rra = ra[l];
      iind = ind[l];
    } else {
      rra = ra[ir];
      iind = ind[ir];
      ra[ir] = ra[1];
      ind[ir] = ind[1];
      ir = ir - 1;
      if (ir == 1) {
        ra[1] = rra;
        ind[1] = iind;
        break;
      }
    }
    i = l;
    j = l + l;
    while (j <= ir) {
      if (j < ir) {
        if (std::fabs(ra[j] - ra[j + 1]) >= eps) {
          if (ra[j] < ra[j + 1]) j = j + 1;
        } else {
          if (ind[j] < ind[j + 1]) j = j + 1;
        }
      }
      if (std::fabs(rra - ra[j]) >= eps) {
        if (rra < ra[j]) {
          ra[i] = ra[j];
          ind[i] = ind[j];
          i = j;
          j = j + j;
        } else {
          j = ir + 1;
        }
      } else {
        if (iind < ind[j]) {
          ra[i] = ra[j];
          ind[i] = ind[j];
          i = j;
          j = j + j;
        } else {
          j = ir + 1;
        }
      }
    }
    ra[i] = rra;
    ind[i] = iind;
  }
}

// a1: gk_sort, Modules/qe_gksort.f90:44-94.  g is g(3,ngm) in 2pi/alat units,
// igk is filled 1-based.  Returns 0, or -1 when ngk exceeds npwx, or -2 when
// the G list ends before |G| leaves the k+G sphere (the reference's "Unexpected
// exit from do-loop").
int orc_gk_sort(const double* k, int npwx, int ngm, const double* g, double ecut, int* ngk_out,
                int* igk, double* gk) {
  const double eps8 = 1.0e-8;
  double kk = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
  double q2x = std::sqrt(kk) + std::sqrt(ecut);
  q2x = q2x * q2x;
  int ngk = 0;
  for (int i = 0; i < npwx; ++i) {
    igk[i] = 0;
    gk[i] = 0.0;
  }
  int ng;
  bool exited = false;
  for (ng = 1; ng <= ngm; ++ng) {
    const double* gg = g + 3 * (ng - 1);
    double a = k[0] + gg[0], b = k[1] + gg[1], c = k[2] + gg[2];
    double q = a * a + b * b + c * c;
    if (q <= eps8) q = 0.0;
    if (q <= ecut) {
      ngk = ngk + 1;
      if (ngk > npwx) return -1;
      gk[ngk - 1] = q;
      igk[ngk - 1] = ng;
    } else {
      double g2 = gg[0] * gg[0] + gg[1] * gg[1] + gg[2] * gg[2];
      if (g2 > (q2x + eps8)) {
        exited = true;
        break;
      }
    }
  }
  if (!exited) return -2;
  orc_hpsort_eps(ngk, gk, igk, eps8);
  for (int nk = 0; nk < ngk; ++nk) {
    const double* gg = g + 3 * (igk[nk] - 1);
    double a = k[0] + gg[0], b = k[1] + gg[1], c = k[2] + gg[2];
    gk[nk] = a * a + b * b + c * c;
  }
  *ngk_out = ngk;
  return 0;
}

// ---------------------------------------------------------------------------
// Helpers for the Fortran layouts.
static inline double Rm(const double* R, int isym1, int i1, int j1) {
  return R[(isym1 - 1) + 48 * ((i1 - 1) + 3 * (j1 - 1))];
}
static inline const double* Gv(const OrcSystem* s, int ig1) { return s->G + 3 * (ig1 - 1); }
static inline int igk_at(const OrcSystem* s, int i1, int kibz1) {
  return s->igk ? s->igk[(i1 - 1) + s->npwx * (kibz1 - 1)] : i1;
}
static inline cplx coef(const OrcSystem* s, int i1, int band1, int kibz1) {
  size_t off = (size_t)(i1 - 1) + (size_t)s->npwx * ((size_t)(band1 - 1) + (size_t)s->nbnd * (size_t)(kibz1 - 1));
  return cplx(s->coeff[2 * off], s->coeff[2 * off + 1]);
}
static inline double Eat(const OrcSystem* s, int kibz1, int band1) {
  return s->E[(kibz1 - 1) + s->nks * (band1 - 1)];
}

// Number of coefficients summed per band for IBZ point K1 (NGd in the legacy
// drivers, npw(K1) in the igk-aware vertices of Modules/vertices.f90:88-189).
static inline int nsum_of(const OrcSystem* s, const OrcParams* p, int K1) {
  return s->igk ? s->npw[K1 - 1] : p->ngd;
}

// a2: Gfast for one FBZ k (0-based ik).  Sloss.f90:905-944 / Optabs.f90:1399-1448
// (float-eps linear search; first match wins; NG2+1 when absent).  In igk mode
// the candidates are G(:,igk(iG2,K2)) as in vertices.f90:122-168.
void orc_gfast(const OrcSystem* s, const OrcParams* p, int ik, int* gfast) {
  int K1 = s->K1[ik], K2 = s->K2[ik], R1 = s->R1[ik], R2 = s->R2[ik], iG0 = s->iG0[ik];
  int NG2 = s->npw[K2 - 1];
  int nsum = nsum_of(s, p, K1);
  int iGfast = 0;
  for (int iG = 1; iG <= s->nlf; ++iG) {
    const double* glf = s->Glf + 3 * (iG - 1);
    for (int iG1 = 1; iG1 <= nsum; ++iG1) {
      const double* g1 = Gv(s, igk_at(s, iG1, K1));
      double k11 = Rm(s->R, R1, 1, 1) * g1[0] + Rm(s->R, R1, 1, 2) * g1[1] + Rm(s->R, R1, 1, 3) * g1[2];
      double k22 = Rm(s->R, R1, 2, 1) * g1[0] + Rm(s->R, R1, 2, 2) * g1[1] + Rm(s->R, R1, 2, 3) * g1[2];
      double k33 = Rm(s->R, R1, 3, 1) * g1[0] + Rm(s->R, R1, 3, 2) * g1[1] + Rm(s->R, R1, 3, 3) * g1[2];
      const double* g0 = Gv(s, iG0);
      k11 = k11 + glf[0] + g0[0];
      k22 = k22 + glf[1] + g0[1];
      k33 = k33 + glf[2] + g0[2];
      double gx = Rm(s->RI, R2, 1, 1) * k11 + Rm(s->RI, R2, 1, 2) * k22 + Rm(s->RI, R2, 1, 3) * k33;
      double gy = Rm(s->RI, R2, 2, 1) * k11 + Rm(s->RI, R2, 2, 2) * k22 + Rm(s->RI, R2, 2, 3) * k33;
      double gz = Rm(s->RI, R2, 3, 1) * k11 + Rm(s->RI, R2, 3, 2) * k22 + Rm(s->RI, R2, 3, 3) * k33;
      int hit = NG2 + 1;
      for (int iG2 = 1; iG2 <= NG2; ++iG2) {
        const double* g2 = Gv(s, igk_at(s, iG2, K2));
        if (std::fabs(g2[0] - gx) < p->eps && std::fabs(g2[1] - gy) < p->eps &&
            std::fabs(g2[2] - gz) < p->eps) {
          hit = iG2;
          break;
        }
      }
      gfast[iGfast++] = hit;
    }
  }
}

// a3: charge vertex genMnmK1K2, Sloss.f90:883-952 (igk-aware form vertices.f90:88-189).
static void vertex_charge(const OrcSystem* s, const OrcParams* p, int ik, int n, int m, const int* gfast,
                          cplx* M) {
  int K1 = s->K1[ik], K2 = s->K2[ik];
  int NG2 = s->npw[K2 - 1];
  int nsum = nsum_of(s, p, K1);
  int iGfast = 0;
  for (int iG = 0; iG < s->nlf; ++iG) {
    cplx acc(0.0, 0.0);
    for (int iG1 = 1; iG1 <= nsum; ++iG1) {
      int iG2 = gfast[iGfast++];
      if (iG2 <= NG2) acc = acc + std::conj(coef(s, iG1, n, K1)) * coef(s, iG2, m, K2);
    }
    M[iG] = acc;
  }
}

// a4: current vertex genStrujniVrhovi, Optabs.f90:1354-1472.
static void vertex_current(const OrcSystem* s, const OrcParams* p, int ik, int n, int m, const int* gfast,
                           cplx* M, cplx* M2) {
  int K1 = s->K1[ik], K2 = s->K2[ik], R1 = s->R1[ik];
  int NG2 = s->npw[K2 - 1];
  int nsum = nsum_of(s, p, K1);
  const double* kv = s->ktot + 3 * ik;
  int iGfast = 0;
  for (int iG = 0; iG < s->nlf; ++iG) {
    const double* glf = s->Glf + 3 * iG;
    cplx acc(0.0, 0.0), acc2(0.0, 0.0);
    for (int iG1 = 1; iG1 <= nsum; ++iG1) {
      const double* g1 = Gv(s, igk_at(s, iG1, K1));
      double k11 = Rm(s->R, R1, 1, 1) * g1[0] + Rm(s->R, R1, 1, 2) * g1[1] + Rm(s->R, R1, 1, 3) * g1[2];
      double k22 = Rm(s->R, R1, 2, 1) * g1[0] + Rm(s->R, R1, 2, 2) * g1[1] + Rm(s->R, R1, 2, 3) * g1[2];
      double k33 = Rm(s->R, R1, 3, 1) * g1[0] + Rm(s->R, R1, 3, 2) * g1[1] + Rm(s->R, R1, 3, 3) * g1[2];
      double jx = (s->q[0] + 2.0 * kv[0] + glf[0] + 2.0 * k11) * p->Gcar;
      double jy = (s->q[1] + 2.0 * kv[1] + glf[1] + 2.0 * k22) * p->Gcar;
      double jz = (s->q[2] + 2.0 * kv[2] + glf[2] + 2.0 * k33) * p->Gcar;
      int iG2 = gfast[iGfast++];
      if (iG2 > NG2) continue;
      cplx c1 = 0.5 * std::conj(coef(s, iG1, n, K1));
      cplx c2 = coef(s, iG2, m, K2);
      switch (p->pol) {
        case ORC_POL_XX: acc = acc + (c1 * jx) * c2; break;
        case ORC_POL_YY: acc = acc + (c1 * jy) * c2; break;
        case ORC_POL_ZZ: acc = acc + (c1 * jz) * c2; break;
        case ORC_POL_YZ:
          acc = acc + (c1 * jy) * c2;
          acc2 = acc2 + (c1 * jz) * c2;
          break;
        default:  // ZY (vertices.f90:281-283)
          acc = acc + (c1 * jz) * c2;
          acc2 = acc2 + (c1 * jy) * c2;
          break;
      }
    }
    M[iG] = acc;
    M2[iG] = (p->pol <= ORC_POL_ZZ) ? acc : acc2;
  }
}

int orc_vertex(const OrcSystem* s, const OrcParams* p, int current, int ik, int n, int m, double* Mout,
               double* M2out) {
  int nsum = nsum_of(s, p, s->K1[ik]);
  std::vector<int> gf((size_t)s->nlf * nsum);
  orc_gfast(s, p, ik, gf.data());
  std::vector<cplx> M(s->nlf), M2(s->nlf);
  if (current)
    vertex_current(s, p, ik, n, m, gf.data(), M.data(), M2.data());
  else {
    vertex_charge(s, p, ik, n, m, gf.data(), M.data());
    M2 = M;
  }
  for (int i = 0; i < s->nlf; ++i) {
    Mout[2 * i] = M[i].real();
    Mout[2 * i + 1] = M[i].imag();
    if (M2out) {
      M2out[2 * i] = M2[i].real();
      M2out[2 * i + 1] = M2[i].imag();
    }
  }
  return 0;
}

static int check_sizes(const OrcSystem* s, const OrcParams* p, int ik) {
  int K1 = s->K1[ik], K2 = s->K2[ik];
  if (!s->igk) {  // "NGd is bigger than NG1/NG2" (Sloss.f90:349-352,378-381)
    if (p->ngd > s->npw[K1 - 1] || p->ngd > s->npw[K2 - 1]) return -1;
  }
  return 0;
}

// a7 + reduction: Sloss S0 (real), Sloss.f90:309-438.  S0(no,nlf,nlf) is
// overwritten (zeroed first, as Sloss.f90:301).
int orc_sloss_s0(const OrcSystem* s, const OrcParams* p, double* S0) {
  const int no = p->no, nlf = s->nlf;
  const size_t nS = (size_t)no * nlf * nlf;
  std::memset(S0, 0, nS * sizeof(double));
  const double pi = 4.0 * std::atan(1.0);
  const double norm = pi * s->ntot * p->Vcell;
  int nk = p->nk_list > 0 ? p->nk_list : s->ntot;
  int err = 0;
#pragma omp parallel num_threads(p->nthreads > 0 ? p->nthreads : omp_get_max_threads())
  {
    std::vector<double> Sp(nS);
    std::vector<int> gfast;
    std::vector<cplx> M(nlf);
#pragma omp for schedule(static)
    for (int ii = 0; ii < nk; ++ii) {
      int ik = p->nk_list > 0 ? p->klist[ii] : ii;
      if (check_sizes(s, p, ik)) {
#pragma omp atomic write
        err = -1;
        continue;
      }
      int K1 = s->K1[ik], K2 = s->K2[ik];
      std::fill(Sp.begin(), Sp.end(), 0.0);
      gfast.assign((size_t)nlf * nsum_of(s, p, K1), 0);
      bool jump = true;  // map rebuilt at the first band pair of every k
      for (int n = 1; n <= p->nocc; ++n) {
        for (int m = p->nocc + 1; m <= s->nbnd; ++m) {
          if (jump) {
            orc_gfast(s, p, ik, gfast.data());
            jump = false;
          }
          vertex_charge(s, p, ik, n, m, gfast.data(), M.data());
          double e1 = Eat(s, K1, n), e2 = Eat(s, K2, m);
          for (int io = 1; io <= no; ++io) {
            double o = (io - 1) * p->domega;
            double dE = o + e1 - e2;
            double Lor = -p->eta / (dE * dE + p->eta * p->eta);
            if (std::fabs(Lor) >= 1.0e-3 / p->eta) {
              for (int jG = 0; jG < nlf; ++jG) {
                for (int iG = 0; iG < nlf; ++iG) {
                  cplx v = ((2.0 * Lor) * M[iG]) * std::conj(M[jG]) / norm;
                  Sp[(io - 1) + (size_t)no * (iG + (size_t)nlf * jG)] -= v.real();
                }
              }
            }
          }
        }
      }
#pragma omp critical(sumS0)
      {
        for (size_t i = 0; i < nS; ++i) S0[i] += Sp[i];
      }
    }
  }
  return err;
}

// a5/a6 + reduction: Optabs S0 (complex, io=-no..no) and Qeff,
// Optabs.f90:291-471.  S0 is complex (2no+1,nlf,nlf), Qeff complex (nlf,nlf).
int orc_optabs_s0(const OrcSystem* s, const OrcParams* p, double* S0d, double* Qd) {
  const int no = p->no, nlf = s->nlf, nw = 2 * no + 1;
  const size_t nS = (size_t)nw * nlf * nlf, nQ = (size_t)nlf * nlf;
  cplx* S0 = reinterpret_cast<cplx*>(S0d);
  cplx* Qeff = reinterpret_cast<cplx*>(Qd);
  std::memset((void*)S0, 0, nS * sizeof(cplx));
  std::memset((void*)Qeff, 0, nQ * sizeof(cplx));
  const double pi = 4.0 * std::atan(1.0);
  const double norm = pi * s->ntot * p->Vcell;
  int nk = p->nk_list > 0 ? p->nk_list : s->ntot;
  int err = 0;
#pragma omp parallel num_threads(p->nthreads > 0 ? p->nthreads : omp_get_max_threads())
  {
    std::vector<cplx> Sp(nS), Qp(nQ), M(nlf), M2(nlf);
    std::vector<int> gfast;
#pragma omp for schedule(static)
    for (int ii = 0; ii < nk; ++ii) {
      int ik = p->nk_list > 0 ? p->klist[ii] : ii;
      if (check_sizes(s, p, ik)) {
#pragma omp atomic write
        err = -1;
        continue;
      }
      int K1 = s->K1[ik], K2 = s->K2[ik];
      std::fill(Sp.begin(), Sp.end(), cplx(0.0, 0.0));
      std::fill(Qp.begin(), Qp.end(), cplx(0.0, 0.0));
      gfast.assign((size_t)nlf * nsum_of(s, p, K1), 0);
      bool jump = true;
      for (int n = 1; n <= s->nbnd; ++n) {
        double expo1, f1;
        orc_occupation(Eat(s, K1, n), p->Efermi, p->T, &expo1, &f1);
        for (int m = 1; m <= s->nbnd; ++m) {
          double expo2, f2;
          orc_occupation(Eat(s, K2, m), p->Efermi, p->T, &expo2, &f2);
          double df = f1 - f2;
          if (!(std::fabs(df) >= p->df_cut || n == m)) continue;
          if (jump) {
            orc_gfast(s, p, ik, gfast.data());
            jump = false;
          }
          vertex_current(s, p, ik, n, m, gfast.data(), M.data(), M2.data());
          double e1 = Eat(s, K1, n), e2 = Eat(s, K2, m);
          if (n != m) {
            for (int io = -no; io <= no; ++io) {
              double o = io * p->domega;
              double dE = o + e1 - e2;
              double Lor = p->eta / (dE * dE + p->eta * p->eta);
              if (std::fabs(Lor) >= p->lor_cut / p->eta) {
                for (int jG = 0; jG < nlf; ++jG)
                  for (int iG = 0; iG < nlf; ++iG)
                    Sp[(io + no) + (size_t)nw * (iG + (size_t)nlf * jG)] -=
                        (((2.0 * df) * Lor) * M[iG]) * std::conj(M2[jG]) / norm;
              }
            }
          } else if (std::fabs(e1 - p->Efermi) <= 10.0 * p->T) {
            double fact = expo1 / ((expo1 + 1.0) * (expo1 + 1.0));
            fact = -fact / p->T;
            for (int jG = 0; jG < nlf; ++jG)
              for (int iG = 0; iG < nlf; ++iG)
                Qp[iG + (size_t)nlf * jG] += ((2.0 * fact) * M[iG]) * std::conj(M2[jG]) / (s->ntot * p->Vcell);
          }
        }
      }
#pragma omp critical(sumS0)
      {
        for (size_t i = 0; i < nS; ++i) S0[i] += Sp[i];
        for (size_t i = 0; i < nQ; ++i) Qeff[i] += Qp[i];
      }
    }
  }
  return err;
}

// ---------------------------------------------------------------------------
// c2: Sloss KK genChi0, Sloss.f90:954-1059.  Note the `if (jo /= io) ... else
// if` chain: the end-point overrides only ever apply at jo == io (where they
// give 0).  S0 real (no,nlf,nlf); chi0 complex (no-1,nlf,nlf).
// Sloss.f90:1050 stores `cmplx(ReChi0,ImChi0)` without a KIND argument, which
// in Fortran yields a default-kind (single precision) complex: the reference's
// chi0 carries float32 rounding.  cmplx_sp=1 emulates that rounding; the
// default (0) keeps full FP64, the evident intent, and is what the CUDA
// library matches.
void orc_kk_sloss(int no, int nlf, double domega, const double* S0, int cmplx_sp, double* chi0d) {
  const double pi = 4.0 * std::atan(1.0);
  cplx* chi0 = reinterpret_cast<cplx*>(chi0d);
#pragma omp parallel for collapse(2) schedule(static)
  for (int jG = 0; jG < nlf; ++jG) {
    for (int iG = 0; iG < nlf; ++iG) {
      const double* s = S0 + (size_t)no * (iG + (size_t)nlf * jG) - 1;  // s[jo], jo=1..no
      for (int io = 1; io <= no - 1; ++io) {
        double oi = (io - 1) * domega;
        double Re = 0.0, fact = 0.0;
        if (io == 1) {
          for (int jo = 2; jo <= no; ++jo) {
            double oj = (jo - 1) * domega;
            fact = domega / oj;
            if (jo == 2) fact = 3.0 / 2.0;
            else if (jo == no) fact = 0.5 * domega / oj;
            Re = Re + fact * s[jo];
          }
          Re = -2.0 * Re;
        } else {
          for (int jo = 1; jo <= no; ++jo) {
            double oj = (jo - 1) * domega;
            if (jo != io) fact = domega / (oi - oj);
            else fact = 0.0;  // every branch's else-if chain lands on 0 at jo == io
            Re = Re + fact * s[jo];
            fact = domega / (oi + oj);
            if (jo == 1 || jo == no) fact = 0.5 * domega / (oi + oj);
            Re = Re - fact * s[jo];
          }
        }
        double Im = -pi * s[io];
        if (cmplx_sp) {
          Re = (double)(float)Re;
          Im = (double)(float)Im;
        }
        chi0[(io - 1) + (size_t)(no - 1) * (iG + (size_t)nlf * jG)] = cplx(Re, Im);
      }
    }
  }
}

// c1: Optabs KK genReChi0 / genImChi0, Optabs.f90:1112-1318.  Independent
// `if`s: the end-point overrides apply.  S0 complex (-no:no,nlf,nlf); chi0
// complex (no-1,nlf,nlf) holding (ReChi0, ImChi0).
static double kk_c1_fact_minus(int io, int no, int jo, double oi, double oj, double domega, double prev) {
  double fact = prev;
  if (io == 2) {
    if (jo != io) fact = domega / (oi - oj);
    if (jo == 1) fact = 1.0;
    else if (jo == 2) fact = 0.0;
    else if (jo == 3) fact = -3.0 / 2.0;
    else if (jo == no) fact = 0.5 * domega / (oi - oj);
  } else if (io == no - 1) {
    if (jo != io) fact = domega / (oi - oj);
    if (jo == 1) fact = 0.5 * domega / (oi - oj);
    else if (jo == no - 2) fact = 3.0 / 2.0;
    else if (jo == no - 1) fact = 0.0;
    else if (jo == no) fact = -1.0;
  } else {
    if (jo != io) fact = domega / (oi - oj);
    if (jo == 1) fact = 0.5 * domega / (oi - oj);
    else if (jo == io - 1) fact = 3.0 / 2.0;
    else if (jo == io) fact = 0.0;
    else if (jo == io + 1) fact = -3.0 / 2.0;
    else if (jo == no) fact = 0.5 * domega / (oi - oj);
  }
  return fact;
}

void orc_kk_optabs(int no, int nlf, double domega, const double* S0d, double* chi0d) {
  const double pi = 4.0 * std::atan(1.0);
  const cplx* S0 = reinterpret_cast<const cplx*>(S0d);
  cplx* chi0 = reinterpret_cast<cplx*>(chi0d);
  const int nw = 2 * no + 1;
#pragma omp parallel for collapse(2) schedule(static)
  for (int jG = 0; jG < nlf; ++jG) {
    for (int iG = 0; iG < nlf; ++iG) {
      const cplx* s = S0 + (size_t)nw * (iG + (size_t)nlf * jG) + no;  // s[j], j=-no..no
      for (int io = 1; io <= no - 1; ++io) {
        double oi = (io - 1) * domega;
        double Re = 0.0, Im = 0.0;
        if (io == 1) {
          for (int jo = 2; jo <= no; ++jo) {
            double oj = (jo - 1) * domega;
            double fact = domega / oj;
            if (jo == 2) fact = 3.0 / 2.0;
            else if (jo == no) fact = 0.5 * domega / oj;
            Re = Re + fact * (s[-jo + 1].real() - s[jo - 1].real());
            Im = Im + fact * (s[-jo + 1].imag() - s[jo - 1].imag());
          }
        } else {
          // Fortran keeps `fact` from the previous jo when no rule fires; the
          // rules above always fire at jo == io, so the carried value never
          // reaches the sum -- it is tracked anyway.
          double fact = 0.0;
          for (int jo = 1; jo <= no; ++jo) {
            double oj = (jo - 1) * domega;
            fact = kk_c1_fact_minus(io, no, jo, oi, oj, domega, fact);
            Re = Re + fact * s[jo - 1].real();
            Im = Im + fact * s[jo - 1].imag();
            double fp = domega / (oi + oj);
            if (jo == 1 || jo == no) fp = 0.5 * domega / (oi + oj);
            Re = Re + fp * s[-jo + 1].real();
            Im = Im + fp * s[-jo + 1].imag();
            fact = fp;
          }
        }
        Re = Re + pi * s[io - 1].imag();
        Im = Im - pi * s[io - 1].real();
        chi0[(io - 1) + (size_t)(no - 1) * (iG + (size_t)nlf * jG)] = cplx(Re, Im);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// d1: genV, Sloss.f90:1173-1208.  q (2pi/a0 units) and Glf (2pi/a0 units) are
// converted with Gcar inside, as Sloss.f90:444-447 does before the call.
void orc_genV(int nlf, double eps, const double* q, const double* Glf, const int* parG, double Gcar,
              double c0, double* V) {
  const double pi = 4.0 * std::atan(1.0);
  double qx = Gcar * q[0], qy = Gcar * q[1];
  for (int iG = 0; iG < nlf; ++iG) {
    double gvx = Gcar * Glf[3 * iG], gvy = Gcar * Glf[3 * iG + 1], gvz = Gcar * Glf[3 * iG + 2];
    double Gabs = std::sqrt((qx + gvx) * (qx + gvx) + (qy + gvy) * (qy + gvy));
    if (Gabs == 0.0) Gabs = eps;
    for (int jG = 0; jG < nlf; ++jG) {
      double v = 0.0;
      double gjz = Gcar * Glf[3 * jG + 2];
      if (Glf[3 * jG] == Glf[3 * iG] && Glf[3 * jG + 1] == Glf[3 * iG + 1]) {
        v = 4.0 * pi * (1.0 - std::exp(-Gabs * c0)) / (Gabs * c0);
        v = v * (Gabs * Gabs - gvz * gjz);
        v = v / (Gabs * Gabs + gvz * gvz);
        v = v / (Gabs * Gabs + gjz * gjz);
        v = -(double)parG[iG] * (double)parG[jG] * v;
        if (Glf[3 * jG + 2] == Glf[3 * iG + 2]) v = 4.0 * pi / (Gabs * Gabs + gvz * gvz) + v;
      }
      V[iG + (size_t)nlf * jG] = v;
    }
  }
}

// d3: Gauss-Jordan inverse with full pivoting, W/gjel.f:1-91, in place on
// a(n,n) (Fortran layout).  The uninitialised right-hand side of the caller
// never feeds into `a` and is not carried.  Returns 0, 1 for the "singular
// matrix" stop (repeated pivot), 2 when a zero pivot was met (the reference
// prints and continues).
int orc_gjel(double* ad, int n) {
  cplx* a = reinterpret_cast<cplx*>(ad);
  auto A = [&](int i1, int j1) -> cplx& { return a[(i1 - 1) + (size_t)n * (j1 - 1)]; };
  std::vector<int> ipiv(n + 1, 0), indxr(n + 1), indxc(n + 1);
  int irow = 0, icol = 0, rc = 0;
  for (int i = 1; i <= n; ++i) {
    double big = 0.0;
    for (int j = 1; j <= n; ++j) {
      if (ipiv[j] != 1) {
        for (int k = 1; k <= n; ++k) {
          if (ipiv[k] == 0) {
            if (std::abs(A(j, k)) >= big) {
              big = std::abs(A(j, k));
              irow = j;
              icol = k;
            }
          } else if (ipiv[k] > 1) {
            return 1;
          }
        }
      }
    }
    ipiv[icol] = ipiv[icol] + 1;
    if (irow != icol) {
      for (int l = 1; l <= n; ++l) std::swap(A(irow, l), A(icol, l));
    }
    indxr[i] = irow;
    indxc[i] = icol;
    if (A(icol, icol) == cplx(0.0, 0.0)) rc = 2;
    cplx pivinv = cplx(1.0, 0.0) / A(icol, icol);
    A(icol, icol) = cplx(1.0, 0.0);
    for (int l = 1; l <= n; ++l) A(icol, l) = A(icol, l) * pivinv;
    for (int ll = 1; ll <= n; ++ll) {
      if (ll != icol) {
        cplx dum = A(ll, icol);
        A(ll, icol) = cplx(0.0, 0.0);
        for (int l = 1; l <= n; ++l) A(ll, l) = A(ll, l) - A(icol, l) * dum;
      }
    }
  }
  for (int l = n; l >= 1; --l) {
    if (indxr[l] != indxc[l]) {
      for (int k = 1; k <= n; ++k) std::swap(A(k, indxr[l]), A(k, indxc[l]));
    }
  }
  return rc;
}

// d2-d5 for every io=1..no-1: eps = I - chi0*V (genDielectricEpsilon,
// Sloss.f90:1210-1234), gjel, chi = eps^-1 chi0 (genChi, :1236-1253),
// WT = V + V chi V (genWT, :1255-1277; 4-deep loop unless fast_wt).
// chi0, WT, epsinv complex (no-1,nlf,nlf) with io fastest; epsinv may be NULL.
int orc_dyson(int no, int nlf, const double* chi0d, const double* V, int fast_wt, int nthreads, double* WTd,
              double* epsinvd) {
  const cplx* chi0 = reinterpret_cast<const cplx*>(chi0d);
  cplx* WT = reinterpret_cast<cplx*>(WTd);
  cplx* epsinv = reinterpret_cast<cplx*>(epsinvd);
  const int nwo = no - 1;
  int rc_all = 0;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
  for (int io = 1; io <= nwo; ++io) {
    std::vector<cplx> C((size_t)nlf * nlf), Ep((size_t)nlf * nlf), Ch((size_t)nlf * nlf), T1;
    for (int j = 0; j < nlf; ++j)
      for (int i = 0; i < nlf; ++i) C[i + (size_t)nlf * j] = chi0[(io - 1) + (size_t)nwo * (i + (size_t)nlf * j)];
    for (int i = 0; i < nlf; ++i) {
      for (int j = 0; j < nlf; ++j) {
        cplx d = (i == j) ? cplx(1.0, 0.0) : cplx(0.0, 0.0);
        for (int k = 0; k < nlf; ++k) d = d - C[i + (size_t)nlf * k] * V[k + (size_t)nlf * j];
        Ep[i + (size_t)nlf * j] = d;
      }
    }
    int rc = orc_gjel(reinterpret_cast<double*>(Ep.data()), nlf);
    if (rc == 1) {
#pragma omp atomic write
      rc_all = 1;
    }
    for (int i = 0; i < nlf; ++i)
      for (int j = 0; j < nlf; ++j) {
        cplx d(0.0, 0.0);
        for (int k = 0; k < nlf; ++k) d = d + Ep[i + (size_t)nlf * k] * C[k + (size_t)nlf * j];
        Ch[i + (size_t)nlf * j] = d;
      }
    if (fast_wt) {
      T1.assign((size_t)nlf * nlf, cplx(0.0, 0.0));
      for (int i = 0; i < nlf; ++i)
        for (int k2 = 0; k2 < nlf; ++k2) {
          cplx d(0.0, 0.0);
          for (int k1 = 0; k1 < nlf; ++k1) d = d + V[i + (size_t)nlf * k1] * Ch[k1 + (size_t)nlf * k2];
          T1[i + (size_t)nlf * k2] = d;
        }
    }
    for (int i = 0; i < nlf; ++i)
      for (int j = 0; j < nlf; ++j) {
        cplx w(0.0, 0.0);
        if (fast_wt) {
          for (int k2 = 0; k2 < nlf; ++k2) w = w + T1[i + (size_t)nlf * k2] * V[k2 + (size_t)nlf * j];
        } else {
          for (int k1 = 0; k1 < nlf; ++k1)
            for (int k2 = 0; k2 < nlf; ++k2)
              w = w + (V[i + (size_t)nlf * k1] * Ch[k1 + (size_t)nlf * k2]) * V[k2 + (size_t)nlf * j];
        }
        WT[(io - 1) + (size_t)nwo * (i + (size_t)nlf * j)] = V[i + (size_t)nlf * j] + w;
        if (epsinv) epsinv[(io - 1) + (size_t)nwo * (i + (size_t)nlf * j)] = Ep[i + (size_t)nlf * j];
      }
  }
  return rc_all;
}

}  // extern "C"
