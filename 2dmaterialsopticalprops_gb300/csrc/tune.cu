// tune.cu -- autotuner of the mixed-path vertex and accumulation tiles.
//
// No counterpart in the reference (its vertices are one CPU loop).  For the
// chi0 call described by args, on the context's current k map and q, every
// candidate configuration of the tensor-core vertex kernel is run (twice: the
// first run builds the index maps and buffers) and its vertex-stage time is
// taken from the stage events; the fastest is kept in the context's table
// under (mode, nbnd, nocc, NGloc / 32) and applies to later rpa_chi0 calls of
// that shape.  Candidates: the width of the sequential-side band windows (16,
// 32, and 48 and 64 for charge vertices) and, for charge vertices, the gathered side
// (occupied bands through the inverse Gfast map, or empty bands through
// Gfast).  The configurations compute the same sums in different tilings, so
// results agree to the mixed path's rounding.
// Then, with the best vertex configuration, every tile variant of the
// warp-specialised S0 accumulation (G-tile rows gb, frequency rows per CTA
// nio; for S0 with M2 = M) is run the same way and timed by its stage event;
// the fastest is kept under (S0 kind, NGloc, nw / 64).  The tables are
// exported and imported as JSON text:
//   {"vertex": [{"mode": 0, "nbnd": 30, "nocc": 8, "nlf32": 2, "ymax": 32, "swap": 1, "ms": 4.21}, ...],
//    "accum": [{"cplx": 0, "nlf": 91, "nw64": 10, "gb": 96, "nio": 2, "ms": 3.10}, ...]}

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "rpa_internal.cuh"

using namespace rpa;

extern "C" {

int rpa_autotune(rpa_ctx* c, const rpa_chi0_args* a, double* best_ms) {
  if (!c || !a) return fail(c, RPA_EINVAL, "rpa_autotune: bad arguments");
  if (c->precision != RPA_PREC_MIXED || c->vertex_kind != 0)
    return fail(c, RPA_ESTATE, "rpa_autotune: tunes the mixed-path tensor-core vertices only");
  struct Cand {
    int ymax, swap;
  };
  std::vector<Cand> cands;
  if (a->mode == RPA_MODE_CURRENT) {
    cands = {{32, -1}, {16, -1}};
  } else {
    for (int sw : {1, 0}) {
      if (sw == 1 && c->legacy) continue;
      for (int y : {64, 48, 32, 16}) cands.push_back({y, sw});
    }
  }
  rpa_ctx::VtxTune best;
  best.ms = 1e300;
  int rc = RPA_OK;
  c->vt_forced = true;
  for (const Cand& k : cands) {
    c->vt_cur.ymax = k.ymax;
    c->vt_cur.swap = k.swap;
    double ms = 0.0;
    for (int rep = 0; rep < 2 && rc == RPA_OK; ++rep) {
      rc = rpa_chi0(c, a, nullptr, nullptr);
      ms = c->stage_ms[1];
    }
    if (rc != RPA_OK) break;
    if (ms < best.ms) {
      best.ymax = k.ymax;
      best.swap = k.swap;
      best.ms = ms;
    }
  }
  c->vt_forced = false;
  c->vt_cur = rpa_ctx::VtxTune();
  if (rc != RPA_OK) return rc;
  c->vt_table[vtx_tune_key(a->mode, c->nbnd, a->mode == RPA_MODE_CHARGE ? a->nocc : 0, c->nlf)] = best;
  if (best_ms) *best_ms = best.ms;
  // accumulation tiles (the warp-specialised kernel; S0 with M2 = M)
  const bool cplx = a->mode == RPA_MODE_CURRENT;
  const bool two = cplx && (a->pol == RPA_POL_YZ || a->pol == RPA_POL_ZY);
  if (two || !c->split_f16 || c->tc_seg != 1) return RPA_OK;
  int gbs[16], nios[16];
  const int nv = std::min(acc_variant_list(cplx, gbs, nios, 16), 16);
  const rpa_ctx::AccTune saved = c->acc_force;
  rpa_ctx::AccTune ab;
  ab.ms = 1e300;
  for (int i = 0; i < nv && rc == RPA_OK; ++i) {
    c->acc_force.gb = gbs[i];
    c->acc_force.nio = nios[i];
    double ms = 0.0;
    for (int rep = 0; rep < 2 && rc == RPA_OK; ++rep) {
      rc = rpa_chi0(c, a, nullptr, nullptr);
      ms = c->stage_ms[2];
    }
    if (rc == RPA_OK && ms < ab.ms) {
      ab.gb = gbs[i];
      ab.nio = nios[i];
      ab.ms = ms;
    }
  }
  c->acc_force = saved;
  if (rc != RPA_OK) return rc;
  const int nw = cplx ? 2 * a->no + 1 : a->no;
  c->acc_table[acc_tune_key(cplx, c->nlf, nw)] = ab;
  return RPA_OK;
}

int rpa_tune_export(const rpa_ctx* c, char* buf, int cap, int* len) {
  if (!c || !len) return fail(nullptr, RPA_EINVAL, "rpa_tune_export: bad arguments");
  std::string s = "{\"vertex\": [";
  bool first = true;
  for (const auto& e : c->vt_table) {
    const long long k = e.first;
    char item[256];
    std::snprintf(item, sizeof item,
                  "%s{\"mode\": %d, \"nbnd\": %d, \"nocc\": %d, \"nlf32\": %d, \"ymax\": %d, \"swap\": %d, \"ms\": %.6g}",
                  first ? "" : ", ", (int)(k & 15), (int)((k >> 4) & 0xffff), (int)((k >> 20) & 0xffff),
                  (int)(k >> 36), e.second.ymax, e.second.swap, e.second.ms);
    s += item;
    first = false;
  }
  s += "], \"accum\": [";
  first = true;
  for (const auto& e : c->acc_table) {
    const long long k = e.first;
    char item[256];
    std::snprintf(item, sizeof item, "%s{\"cplx\": %d, \"nlf\": %d, \"nw64\": %d, \"gb\": %d, \"nio\": %d, \"ms\": %.6g}",
                  first ? "" : ", ", (int)(k & 1), (int)((k >> 1) & 0x7fff), (int)(k >> 16), e.second.gb, e.second.nio,
                  e.second.ms);
    s += item;
    first = false;
  }
  s += "]}";
  *len = (int)s.size() + 1;
  if (!buf) return RPA_OK;
  if (cap < *len) return fail(const_cast<rpa_ctx*>(c), RPA_EINVAL, "rpa_tune_export: buffer of %d bytes, %d needed", cap, *len);
  std::memcpy(buf, s.c_str(), (size_t)*len);
  return RPA_OK;
}

// value of "name": <number> inside one JSON object [p, q)
static bool field(const char* p, const char* q, const char* name, double* v) {
  const std::string key = std::string("\"") + name + "\"";
  const char* f = std::strstr(p, key.c_str());
  if (!f || f >= q) return false;
  f = std::strchr(f + key.size(), ':');
  if (!f || f >= q) return false;
  char* end = nullptr;
  *v = std::strtod(f + 1, &end);
  return end && end != f + 1 && end <= q;
}

int rpa_tune_import(rpa_ctx* c, const char* json) {
  if (!c || !json) return fail(c, RPA_EINVAL, "rpa_tune_import: bad arguments");
  const char* p = std::strstr(json, "\"vertex\"");
  if (!p) return fail(c, RPA_EINVAL, "rpa_tune_import: no \"vertex\" list");
  p = std::strchr(p, '[');
  const char* end = p ? std::strchr(p, ']') : nullptr;
  if (!p || !end) return fail(c, RPA_EINVAL, "rpa_tune_import: malformed list");
  std::map<long long, rpa_ctx::VtxTune> table;
  for (const char* o = std::strchr(p, '{'); o && o < end; o = std::strchr(o + 1, '{')) {
    const char* q = std::strchr(o, '}');
    if (!q || q > end) return fail(c, RPA_EINVAL, "rpa_tune_import: malformed entry");
    double mode, nbnd, nocc, nlf32, ymax, swap, ms = 0.0;
    if (!field(o, q, "mode", &mode) || !field(o, q, "nbnd", &nbnd) || !field(o, q, "nocc", &nocc) ||
        !field(o, q, "nlf32", &nlf32) || !field(o, q, "ymax", &ymax) || !field(o, q, "swap", &swap))
      return fail(c, RPA_EINVAL, "rpa_tune_import: entry without mode/nbnd/nocc/nlf32/ymax/swap");
    field(o, q, "ms", &ms);
    if (!(ymax == 0 || ymax == 16 || ymax == 32 || ymax == 48 || ymax == 64) || swap < -1 || swap > 1)
      return fail(c, RPA_EINVAL, "rpa_tune_import: ymax %g / swap %g not a configuration", ymax, swap);
    rpa_ctx::VtxTune v;
    v.ymax = (int)ymax;
    v.swap = (int)swap;
    v.ms = ms;
    table[vtx_tune_key((int)mode, (int)nbnd, (int)nocc, 32 * (int)nlf32)] = v;
  }
  // the accumulation list is optional (tables written before it existed)
  std::map<long long, rpa_ctx::AccTune> atable;
  const char* pa = std::strstr(json, "\"accum\"");
  if (pa) {
    pa = std::strchr(pa, '[');
    const char* ea = pa ? std::strchr(pa, ']') : nullptr;
    if (!pa || !ea) return fail(c, RPA_EINVAL, "rpa_tune_import: malformed accum list");
    int gbs[16], nios[16];
    const int nvc = acc_variant_list(true, gbs, nios, 16);
    int gbr[16], nior[16];
    const int nvr = acc_variant_list(false, gbr, nior, 16);
    for (const char* o = std::strchr(pa, '{'); o && o < ea; o = std::strchr(o + 1, '{')) {
      const char* q = std::strchr(o, '}');
      if (!q || q > ea) return fail(c, RPA_EINVAL, "rpa_tune_import: malformed accum entry");
      double cplx, nlf, nw64, gb, nio, ms = 0.0;
      if (!field(o, q, "cplx", &cplx) || !field(o, q, "nlf", &nlf) || !field(o, q, "nw64", &nw64) ||
          !field(o, q, "gb", &gb) || !field(o, q, "nio", &nio))
        return fail(c, RPA_EINVAL, "rpa_tune_import: accum entry without cplx/nlf/nw64/gb/nio");
      field(o, q, "ms", &ms);
      bool known = false;
      const int n = cplx != 0 ? nvc : nvr;
      for (int i = 0; i < n; ++i)
        known = known || (cplx != 0 ? (gbs[i] == (int)gb && nios[i] == (int)nio) : (gbr[i] == (int)gb && nior[i] == (int)nio));
      if (!known) return fail(c, RPA_EINVAL, "rpa_tune_import: accumulation tile (%g, %g) not a variant", gb, nio);
      rpa_ctx::AccTune v;
      v.gb = (int)gb;
      v.nio = (int)nio;
      v.ms = ms;
      atable[acc_tune_key(cplx != 0, (int)nlf, 64 * (int)nw64)] = v;
    }
  }
  c->vt_table = table;
  c->acc_table = atable;
  return RPA_OK;
}

}  // extern "C"
