// tune.cu -- autotuner of the mixed-path vertex configuration.
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
// results agree to the mixed path's rounding.  The table is exported and
// imported as JSON text:
//   {"vertex": [{"mode": 0, "nbnd": 30, "nocc": 8, "nlf32": 2, "ymax": 32, "swap": 1, "ms": 4.21}, ...]}

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
  c->vt_table = table;
  return RPA_OK;
}

}  // extern "C"
