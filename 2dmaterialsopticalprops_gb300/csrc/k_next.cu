// k_next.cu -- the consumers right after the hot path in the two drivers:
//   * the current-response assembly of Optabs calc = 2 (Optabs.f90:575-614):
//     Pi = chi0 + Pi_dia + Qeff oi / (oi + i eta_intra), the Pi_11 spectrum and
//     the inter- and intraband conductivities;
//   * the Kramers-Kronig transform of the screened interaction and its
//     self-check in Sloss (Sloss.f90:486-534, genW1W2 at :1062-1171,
//     writeKramKron_Qi at :1603-1641).
// Both run on the device data the hot path leaves there (chi0, Qeff, S0, W, V).

#include <cmath>
#include <vector>

#include "rpa_internal.cuh"

namespace rpa {

// Pi(io, p) = chi0(io, p) - Re chi0(1, p) + Qeff(p) oi / (oi + i eta), io0 = io - 1
__global__ void k_pi(const double2* __restrict__ chi0, const double2* __restrict__ Q, double2* __restrict__ Pi,
                     int nwo, int np, double domega, double eta) {
  const size_t n = (size_t)nwo * np;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int io0 = (int)(e / np), p = (int)(e % np);
    const double oi = io0 * domega;
    const double2 x = chi0[e];
    const double dia = -chi0[p].x;
    // Qeff * oi / (oi + i eta): (q oi) (oi - i eta) / (oi^2 + eta^2)
    const double2 q = Q[p];
    const double den = oi * oi + eta * eta;
    const double qr = q.x * oi, qi = q.y * oi;
    const double ir = (qr * oi + qi * eta) / den, ii = (qi * oi - qr * eta) / den;
    Pi[e] = make_double2(x.x + dia + ir, x.y + ii);
  }
}

// Spectral function of W for its KK transform, rows jo = 1..no:
// S_W(jo) = -Im WT(jo) / pi for jo < no; row no keeps the chi0 spectral
// function S0(no), which the driver never overwrites (Sloss.f90:486).
__global__ void k_spectral_w(const double2* __restrict__ WT, const double* __restrict__ S0, double* __restrict__ SW,
                             int no, int np) {
  const size_t n = (size_t)no * np;
  const double inv_pi = 0.318309886183790671537767526745028724;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / np);
    SW[e] = r < no - 1 ? -inv_pi * WT[e].y : S0[e];
  }
}

// genW1W2 (Sloss.f90:1062-1171) as two kernel matrices [(no-1) x no]:
// W1 = Km S_W, W2 = Kp S_W.  In every branch of the driver's else-if chain the
// overrides apply only at jo == io, where they set fact = 0.
static void w1w2_matrices(int no, double domega, std::vector<double>& Km, std::vector<double>& Kp) {
  Km.assign((size_t)(no - 1) * no, 0.0);
  Kp.assign((size_t)(no - 1) * no, 0.0);
  for (int io = 1; io <= no - 1; ++io) {
    const double oi = (io - 1) * domega;
    double* rm = Km.data() + (size_t)(io - 1) * no;
    double* rp = Kp.data() + (size_t)(io - 1) * no;
    if (io == 1) {
      // static limit: W1 = -sum fact S0(jo), W2 = -W1
      for (int jo = 2; jo <= no; ++jo) {
        const double oj = (jo - 1) * domega;
        double fact = domega / oj;
        if (jo == 2) fact = 3.0 / 2.0;
        else if (jo == no) fact = 0.5 * domega / oj;
        rm[jo - 1] -= fact;
        rp[jo - 1] += fact;
      }
      continue;
    }
    for (int jo = 1; jo <= no; ++jo) {
      const double oj = (jo - 1) * domega;
      rm[jo - 1] += jo != io ? domega / (oi - oj) : 0.0;
      double fp = domega / (oi + oj);
      if (jo == 1 || jo == no) fp = 0.5 * domega / (oi + oj);
      rp[jo - 1] += fp;
    }
  }
}

static double ev_ms(rpa_ctx* c, int a, int b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev[a], c->ev[b]);
  return ms;
}

}  // namespace rpa

using namespace rpa;

extern "C" {

int rpa_pi(rpa_ctx* c, double eta_intra, double c0, double* pi11_out, double* sigma_out, double* Pi_out) {
  if (!c) return fail(c, RPA_EINVAL, "rpa_pi: ctx is NULL");
  if (!c->have_chi0 || c->last_mode != RPA_MODE_CURRENT)
    return fail(c, RPA_ESTATE, "rpa_pi: needs the Optabs chi0 on the device (rpa_chi0 current + rpa_kk)");
  if (!(eta_intra > 0)) return fail(c, RPA_EINVAL, "rpa_pi: eta_intra must be > 0");
  cudaSetDevice(c->device);
  const int nwo = c->last_no - 1, np = c->nlf * c->nlf;
  RPA_TRY(ensure(c, c->d_tmp, sizeof(double2) * (size_t)nwo * np * 2));
  double2* Pi = c->d_tmp.as<double2>();
  k_pi<<<1024, 256, 0, c->stream>>>(c->d_chi0.as<double2>(), c->d_Q.as<double2>(), Pi, nwo, np, c->last_domega,
                                    eta_intra);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  // Pi_11 per frequency (element p = 0) and Qeff_11
  std::vector<double2> p11(nwo);
  double2 q11;
  RPA_CUDA(c, cudaMemcpy2DAsync(p11.data(), sizeof(double2), Pi, sizeof(double2) * np, sizeof(double2), nwo,
                                cudaMemcpyDeviceToHost, c->stream));
  RPA_CUDA(c, cudaMemcpyAsync(&q11, c->d_Q.p, sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
  if (Pi_out) {
    double* tr = reinterpret_cast<double*>(Pi + (size_t)nwo * np);
    launch_transpose_wp_to_fortran(reinterpret_cast<const double*>(Pi), tr, nwo, np, 2, c->stream);
    RPA_CUDA(c, cudaGetLastError());
    ++c->launches;
    RPA_CUDA(c, cudaMemcpyAsync(Pi_out, tr, sizeof(double2) * (size_t)nwo * np, cudaMemcpyDeviceToHost, c->stream));
  }
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  const double domega = c->last_domega;
  for (int io = 1; io <= nwo; ++io) {
    const double oi = (io - 1) * domega;
    const double2 pt = p11[io - 1];
    if (pi11_out) {
      pi11_out[2 * (io - 1)] = pt.x;
      pi11_out[2 * (io - 1) + 1] = pt.y;
    }
    if (!sigma_out) continue;
    // Pi_intra = Qeff_11 oi / (oi + i eta); Pi_inter is Pi_tot(1,1) as the
    // driver leaves it after its (iG, jG) loop: with the intraband term once
    // Nlf > 1 (it is read after element (1,1) was completed), without it for
    // Nlf = 1 (Optabs.f90:593-597)
    const double den = oi * oi + eta_intra * eta_intra;
    const double qr = q11.x * oi, qi = q11.y * oi;
    const double intra_i = (qi * oi - qr * eta_intra) / den;
    double inter_i = pt.y;
    if (c->nlf == 1) inter_i -= intra_i;
    // sigma = Re(-i c0 Pi / oi) = c0 Im(Pi) / oi, written for io > 1 only
    sigma_out[2 * (io - 1)] = io > 1 ? c0 * inter_i / oi : 0.0;
    sigma_out[2 * (io - 1) + 1] = io > 1 ? c0 * intra_i / oi : 0.0;
  }
  return RPA_OK;
}

int rpa_kk_w(rpa_ctx* c, double* gamma_p_out, double* gamma_m_out, double* check5) {
  if (!c) return fail(c, RPA_EINVAL, "rpa_kk_w: ctx is NULL");
  if (!c->have_W || c->last_mode != RPA_MODE_CHARGE)
    return fail(c, RPA_ESTATE, "rpa_kk_w: needs the Sloss W on the device (rpa_chi0 charge, rpa_kk, rpa_dyson)");
  cudaSetDevice(c->device);
  const int no = c->last_no, nwo = no - 1, np = c->nlf * c->nlf;
  // scratch: S_W [no][np] real, Gamma+ and Gamma- [nwo][np] complex, one transpose buffer
  const size_t sw_bytes = sizeof(double) * (size_t)no * np, g_bytes = sizeof(double2) * (size_t)nwo * np;
  RPA_TRY(ensure(c, c->d_tmp, sw_bytes + 3 * g_bytes + 256));
  double* SW = c->d_tmp.as<double>();
  double2* Gp = reinterpret_cast<double2*>(c->d_tmp.as<char>() + ((sw_bytes + 255) & ~size_t(255)));
  double2* Gm = Gp + (size_t)nwo * np;
  double2* tr = Gm + (size_t)nwo * np;
  cudaEventRecord(c->ev[0], c->stream);
  k_spectral_w<<<1024, 256, 0, c->stream>>>(c->d_WT.as<double2>(), c->d_S.as<double>(), SW, no, np);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  std::vector<double> Km, Kp;
  w1w2_matrices(no, c->last_domega, Km, Kp);
  // Gamma+ = (W1, -pi S_W(io)) = (W1, Im WT); Gamma- = (-W2, 0)
  RPA_TRY(kk_apply_real_fp64(c, c->d_kkw, Km, nwo, no, SW, Gp, np, true));
  for (double& x : Kp) x = -x;
  RPA_TRY(kk_apply_real_fp64(c, c->d_kkw, Kp, nwo, no, SW, Gm, np, false));
  cudaEventRecord(c->ev[1], c->stream);
  // self-check on the (1,1) element (Sloss.f90:515-530)
  std::vector<double2> gp(nwo), gm(nwo), wt(nwo);
  double v11 = 0;
  RPA_CUDA(c, cudaMemcpy2DAsync(gp.data(), sizeof(double2), Gp, sizeof(double2) * np, sizeof(double2), nwo,
                                cudaMemcpyDeviceToHost, c->stream));
  RPA_CUDA(c, cudaMemcpy2DAsync(gm.data(), sizeof(double2), Gm, sizeof(double2) * np, sizeof(double2), nwo,
                                cudaMemcpyDeviceToHost, c->stream));
  RPA_CUDA(c, cudaMemcpy2DAsync(wt.data(), sizeof(double2), c->d_WT.p, sizeof(double2) * np, sizeof(double2), nwo,
                                cudaMemcpyDeviceToHost, c->stream));
  RPA_CUDA(c, cudaMemcpyAsync(&v11, c->d_V.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (gamma_p_out) {
    launch_transpose_wp_to_fortran(reinterpret_cast<const double*>(Gp), reinterpret_cast<double*>(tr), nwo, np, 2,
                                   c->stream);
    RPA_CUDA(c, cudaGetLastError());
    ++c->launches;
    RPA_CUDA(c, cudaMemcpyAsync(gamma_p_out, tr, g_bytes, cudaMemcpyDeviceToHost, c->stream));
    RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  if (gamma_m_out) {
    launch_transpose_wp_to_fortran(reinterpret_cast<const double*>(Gm), reinterpret_cast<double*>(tr), nwo, np, 2,
                                   c->stream);
    RPA_CUDA(c, cudaGetLastError());
    ++c->launches;
    RPA_CUDA(c, cudaMemcpyAsync(gamma_m_out, tr, g_bytes, cudaMemcpyDeviceToHost, c->stream));
  }
  RPA_CUDA(c, cudaStreamSynchronize(c->stream));
  c->stage_ms[3] = ev_ms(c, 0, 1);
  if (check5) {
    double kks = 0, skk = 0;
    const double domega = c->last_domega;
    for (int io = 1; io <= nwo; ++io) {
      const double wind = wt[io - 1].x - v11;
      const double w2kk = -gm[io - 1].x;
      const double windkk = gp[io - 1].x - w2kk;
      const double fact = (io == 1 || io == no - 1) ? 0.5 * domega : domega;
      kks += fact * (windkk - wind) * (windkk - wind);
      skk += fact * wind * wind;
    }
    check5[0] = kks;                           // int (WindKK - Wind)^2
    check5[1] = skk;                           // int Wind^2
    check5[2] = 100.0 * std::fabs(kks / skk);  // relative error, percent
    check5[3] = gp[0].x;                       // real Gamma(o=0,1,1)
    check5[4] = (wt[0].x - v11) / 2.0;         // real[WT(o=0,1,1) - V(1,1)] / 2
  }
  return RPA_OK;
}

}  // extern "C"
