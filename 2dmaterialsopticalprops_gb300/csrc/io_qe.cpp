// io_qe.cpp -- the on-disk formats on either side of the path (host code).
//
//  * QE 6 binary output read by the drivers (Modules/io_qe.f90): the G list of
//    charge-density.dat (loadG, :11-71) and the coefficients of wfc<ik>.dat
//    (loadCs_full, :124-166).  Both are Fortran unformatted sequential files:
//    every record is framed by its byte length as a 4-byte integer before and
//    after the data (records up to 2^31 - 1 bytes; longer ones, which a writer
//    splits into sub-records, are reported as an error).
//      charge-density.dat: (gamma_only, ngm, nspin) | (b1, b2, b3) | mill(3, ngm) | ...
//      wfc<ik>.dat: (ik, xk(3), ispin, gamma_only, scalef) | (ngw, igwx, npol, nbnd) |
//                   (b1, b2, b3) | mill(3, igwx) | evc(npol igwx) for each band
//  * The text files of the Optabs calc = 1 -> 2 hand-over (Chi_RPA/Optabs.f90:
//    482-508 written, :531-559 read back): for io = -no..no an 'omega=' line,
//    then S0(io, iG, jG) for iG outer, jG inner as '(2F15.10)'; the Qeff file
//    holds Qeff(iG, jG) in the same layout.  The reader, like the Fortran
//    formatted read, skips the 'omega=' line and takes each value from its
//    15-character field.
//  * W_Qi of Sloss (writeWT_Qi, W/Sloss.f90:1572-1601): the first frequency of
//    WT only, an 'omega=' line and ((WT(1, iG, jG), jG), iG) as '(10F15.5)'
//    (real and imaginary parts as consecutive values, 10 per line).
// Fixed-point fields follow Fortran F editing: right-aligned, rounded to the
// stated decimals, and all asterisks when the value does not fit the width.
// The 'omega=' line is list-directed output in the reference (its spacing is
// the compiler's); it is written here as " omega= <value in E format> Hartree"
// and is never parsed back.

#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rpa_gpu.h"

namespace rpa {
int fail(rpa_ctx* c, int code, const char* fmt, ...);
}

namespace {

struct File {
  FILE* f = nullptr;
  explicit File(const std::string& path, const char* mode) : f(std::fopen(path.c_str(), mode)) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

// Reads one record of a Fortran unformatted sequential file; data may be NULL
// (skip).  Returns the record length, -1 at end of file, -2 on a bad frame.
long long read_record(FILE* f, std::vector<unsigned char>* data) {
  int32_t head = 0, tail = 0;
  if (std::fread(&head, 4, 1, f) != 1) return -1;
  if (head < 0) return -2;
  if (data) {
    data->resize((size_t)head);
    if (head > 0 && std::fread(data->data(), 1, (size_t)head, f) != (size_t)head) return -2;
  } else if (std::fseek(f, head, SEEK_CUR) != 0) {
    return -2;
  }
  if (std::fread(&tail, 4, 1, f) != 1 || tail != head) return -2;
  return head;
}

template <typename T>
T get(const std::vector<unsigned char>& r, size_t off) {
  T v;
  std::memcpy(&v, r.data() + off, sizeof(T));
  return v;
}

// Fortran Fw.d of x: right-aligned in w characters, asterisks on overflow
void fmt_f(char* out, int w, int d, double x) {
  char buf[64];
  const int n = std::snprintf(buf, sizeof buf, "%*.*f", w, d, x);
  if (n > w || !std::isfinite(x)) {
    std::memset(out, '*', (size_t)w);
  } else {
    std::memcpy(out, buf, (size_t)w);
  }
  out[w] = '\0';
}

// value of a w-character field of a formatted read (blank field -> 0)
bool parse_field(const char* s, int w, double* v) {
  char buf[64];
  std::memcpy(buf, s, (size_t)w);
  buf[w] = '\0';
  char* p = buf;
  while (*p == ' ') ++p;
  if (*p == '\0') {
    *v = 0.0;
    return true;
  }
  char* end = nullptr;
  *v = std::strtod(p, &end);
  while (end && *end == ' ') ++end;
  return end && *end == '\0';
}

std::string wfc_path(const char* savedir, int ik) { return std::string(savedir) + "/wfc" + std::to_string(ik) + ".dat"; }

}  // namespace

using rpa::fail;

extern "C" {

int rpa_qe_read_gvectors(const char* savedir, const double* KC, int max_ng, int* ng, int* miller, double* G,
                         int* parG) {
  if (!savedir || !KC || !ng || !miller || !G || max_ng < 1)
    return fail(nullptr, RPA_EINVAL, "rpa_qe_read_gvectors: bad arguments");
  const std::string path = std::string(savedir) + "/charge-density.dat";
  File fh(path, "rb");
  if (!fh.f) return fail(nullptr, RPA_EINVAL, "Can't open G-vector file %s", path.c_str());
  std::vector<unsigned char> r;
  if (read_record(fh.f, &r) < 12) return fail(nullptr, RPA_EINVAL, "Failed to read NG and Nspin from G-vector file.");
  const int n = get<int32_t>(r, 4);
  if (n < 1) return fail(nullptr, RPA_EINVAL, "G-vector file: NG = %d", n);
  if (n > max_ng) return fail(nullptr, RPA_EINVAL, "G-vector file: NG = %d is above max_ng = %d", n, max_ng);
  if (read_record(fh.f, nullptr) < 0) return fail(nullptr, RPA_EINVAL, "Failed to read the reciprocal axes.");
  if (read_record(fh.f, &r) != 12LL * n) return fail(nullptr, RPA_EINVAL, "Failed to read Miller indices from G-vector file.");
  for (int g = 0; g < n; ++g) {
    int m[3];
    for (int d = 0; d < 3; ++d) m[d] = miller[3 * g + d] = get<int32_t>(r, 12 * (size_t)g + 4 * d);
    // G(n,iG) = sum_m KC(n,m) Gi(m,iG), accumulated from zero in m order
    for (int a = 0; a < 3; ++a) {
      double s = 0.0;
      for (int b = 0; b < 3; ++b) s = s + KC[a + 3 * b] * (double)m[b];
      G[3 * g + a] = s;
    }
    if (parG) parG[g] = m[2];
  }
  *ng = n;
  return RPA_OK;
}

int rpa_qe_wfc_info(const char* savedir, int ik, int* igwx, int* npol, int* nbnd, double* xk) {
  if (!savedir || ik < 1 || !igwx || !npol || !nbnd) return fail(nullptr, RPA_EINVAL, "rpa_qe_wfc_info: bad arguments");
  const std::string path = wfc_path(savedir, ik);
  File fh(path, "rb");
  if (!fh.f) return fail(nullptr, RPA_EINVAL, "Can't open %s", path.c_str());
  std::vector<unsigned char> r;
  if (read_record(fh.f, &r) < 28) return fail(nullptr, RPA_EINVAL, "%s: bad first record", path.c_str());
  if (xk)
    for (int d = 0; d < 3; ++d) xk[d] = get<double>(r, 4 + 8 * (size_t)d);
  if (read_record(fh.f, &r) < 16) return fail(nullptr, RPA_EINVAL, "%s: bad dimension record", path.c_str());
  *igwx = get<int32_t>(r, 4);
  *npol = get<int32_t>(r, 8);
  *nbnd = get<int32_t>(r, 12);
  return RPA_OK;
}

int rpa_qe_read_wfc(const char* savedir, int ik, int npwx, int nbnd, double* coeff, int* miller) {
  if (!savedir || ik < 1 || npwx < 1 || nbnd < 1 || !coeff) return fail(nullptr, RPA_EINVAL, "rpa_qe_read_wfc: bad arguments");
  const std::string path = wfc_path(savedir, ik);
  File fh(path, "rb");
  if (!fh.f) return fail(nullptr, RPA_EINVAL, "Can't open %s", path.c_str());
  std::vector<unsigned char> r;
  if (read_record(fh.f, &r) < 28) return fail(nullptr, RPA_EINVAL, "%s: bad first record", path.c_str());
  if (read_record(fh.f, &r) < 16) return fail(nullptr, RPA_EINVAL, "%s: bad dimension record", path.c_str());
  const int igwx = get<int32_t>(r, 4), npol = get<int32_t>(r, 8), nb = get<int32_t>(r, 12);
  if (npol != 1) return fail(nullptr, RPA_EINVAL, "%s: npol = %d (spinor wavefunctions are not read)", path.c_str(), npol);
  if (igwx > npwx) return fail(nullptr, RPA_EINVAL, "%s: igwx = %d is above npwx = %d", path.c_str(), igwx, npwx);
  if (nbnd > nb)
    return fail(nullptr, RPA_EINVAL, "Looking for band nr. %d but there are only %d bands in the file.", nbnd, nb);
  if (read_record(fh.f, nullptr) < 0) return fail(nullptr, RPA_EINVAL, "%s: bad axes record", path.c_str());
  if (read_record(fh.f, miller ? &r : nullptr) != 12LL * igwx)
    return fail(nullptr, RPA_EINVAL, "%s: bad Miller-index record", path.c_str());
  if (miller)
    for (int e = 0; e < 3 * igwx; ++e) miller[e] = get<int32_t>(r, 4 * (size_t)e);
  for (int b = 0; b < nbnd; ++b) {
    if (read_record(fh.f, &r) != 16LL * igwx) return fail(nullptr, RPA_EINVAL, "%s: bad record of band %d", path.c_str(), b + 1);
    double* dst = coeff + 2 * (size_t)npwx * b;
    std::memcpy(dst, r.data(), 16 * (size_t)igwx);
    std::memset(dst + 2 * (size_t)igwx, 0, 16 * (size_t)(npwx - igwx));
  }
  return RPA_OK;
}

int rpa_write_corrfun(const char* path_s0, const char* path_qeff, int no, int nlf, double domega, const double* S0,
                      const double* Qeff) {
  if (!path_s0 || no < 1 || nlf < 1 || !S0) return fail(nullptr, RPA_EINVAL, "rpa_write_corrfun: bad arguments");
  {
    File fh(path_s0, "w");
    if (!fh.f) return fail(nullptr, RPA_EINVAL, "Can't open %s", path_s0);
    const size_t nw = 2 * (size_t)no + 1;
    char a[32], b[32];
    for (int io = -no; io <= no; ++io) {
      std::fprintf(fh.f, " omega= %23.16E Hartree\n", io * domega);
      for (int iG = 0; iG < nlf; ++iG)
        for (int jG = 0; jG < nlf; ++jG) {
          // S0(-no:no, nlf, nlf) complex, column-major
          const double* v = S0 + 2 * ((size_t)(io + no) + nw * ((size_t)iG + (size_t)nlf * jG));
          fmt_f(a, 15, 10, v[0]);
          fmt_f(b, 15, 10, v[1]);
          std::fprintf(fh.f, "%s%s\n", a, b);
        }
    }
    if (std::ferror(fh.f)) return fail(nullptr, RPA_EINVAL, "write error on %s", path_s0);
  }
  if (path_qeff && Qeff) {
    File fh(path_qeff, "w");
    if (!fh.f) return fail(nullptr, RPA_EINVAL, "Can't open %s", path_qeff);
    char a[32], b[32];
    for (int iG = 0; iG < nlf; ++iG)
      for (int jG = 0; jG < nlf; ++jG) {
        const double* v = Qeff + 2 * ((size_t)iG + (size_t)nlf * jG);
        fmt_f(a, 15, 10, v[0]);
        fmt_f(b, 15, 10, v[1]);
        std::fprintf(fh.f, "%s%s\n", a, b);
      }
    if (std::ferror(fh.f)) return fail(nullptr, RPA_EINVAL, "write error on %s", path_qeff);
  }
  return RPA_OK;
}

int rpa_read_corrfun(const char* path_s0, const char* path_qeff, int no, int nlf, double* S0, double* Qeff) {
  if (!path_s0 || no < 1 || nlf < 1 || !S0) return fail(nullptr, RPA_EINVAL, "rpa_read_corrfun: bad arguments");
  auto read_pairs = [&](FILE* f, double* dst, size_t stride_lo, size_t base, bool skip_headers, const char* path) -> int {
    char line[512];
    const int nblocks = skip_headers ? 2 * no + 1 : 1;
    for (int blk = 0; blk < nblocks; ++blk) {
      if (skip_headers && !std::fgets(line, sizeof line, f))
        return fail(nullptr, RPA_EINVAL, "%s: ends before frequency %d", path, blk - no);
      for (int iG = 0; iG < nlf; ++iG)
        for (int jG = 0; jG < nlf; ++jG) {
          if (!std::fgets(line, sizeof line, f)) return fail(nullptr, RPA_EINVAL, "%s: ends early", path);
          char padded[64];
          std::memset(padded, ' ', 30);
          const size_t L = std::strcspn(line, "\r\n");
          std::memcpy(padded, line, L < 30 ? L : 30);
          double re, im;
          if (!parse_field(padded, 15, &re) || !parse_field(padded + 15, 15, &im))
            return fail(nullptr, RPA_EINVAL, "%s: bad value field", path);
          double* v = dst + 2 * ((size_t)blk * base + stride_lo * ((size_t)iG + (size_t)nlf * jG));
          v[0] = re;
          v[1] = im;
        }
    }
    return RPA_OK;
  };
  {
    File fh(path_s0, "r");
    if (!fh.f) return fail(nullptr, RPA_EINVAL, "Can't open %s", path_s0);
    // S0(io, iG, jG): io fastest (stride 1 per block), (iG, jG) stride 2 no + 1
    const int rc = read_pairs(fh.f, S0, 2 * (size_t)no + 1, 1, true, path_s0);
    if (rc != RPA_OK) return rc;
  }
  if (path_qeff && Qeff) {
    File fh(path_qeff, "r");
    if (!fh.f) return fail(nullptr, RPA_EINVAL, "Can't open %s", path_qeff);
    const int rc = read_pairs(fh.f, Qeff, 1, 0, false, path_qeff);
    if (rc != RPA_OK) return rc;
  }
  return RPA_OK;
}

int rpa_write_wt(const char* path, int no_rows, int nlf, double domega, const double* WT) {
  if (!path || no_rows < 1 || nlf < 1 || !WT) return fail(nullptr, RPA_EINVAL, "rpa_write_wt: bad arguments");
  File fh(path, "w");
  if (!fh.f) return fail(nullptr, RPA_EINVAL, "Can't open %s", path);
  std::fprintf(fh.f, " omega= %23.16E Hartree\n", 0.0 * domega);
  char v[32];
  int col = 0;
  for (int iG = 0; iG < nlf; ++iG)
    for (int jG = 0; jG < nlf; ++jG) {
      // WT(no_rows, nlf, nlf) complex, column-major; the first frequency row
      const double* w = WT + 2 * ((size_t)no_rows * ((size_t)iG + (size_t)nlf * jG));
      for (int part = 0; part < 2; ++part) {
        fmt_f(v, 15, 5, w[part]);
        std::fputs(v, fh.f);
        if (++col == 10) {
          std::fputc('\n', fh.f);
          col = 0;
        }
      }
    }
  if (col) std::fputc('\n', fh.f);
  if (std::ferror(fh.f)) return fail(nullptr, RPA_EINVAL, "write error on %s", path);
  return RPA_OK;
}

}  // extern "C"
