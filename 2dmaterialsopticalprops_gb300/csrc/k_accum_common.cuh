// k_accum_common.cuh -- pieces shared by the tensor-core S0 accumulation
// kernels (k_accum_tc.cu and the warp-specialised k_accum_ws.cuh): the launch
// context, tile constants, the 16-bit operand split, the 128-byte swizzled
// store, the window-start search and double-float addition.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstring>

#include "rpa_internal.cuh"
#include "tc05.cuh"

namespace rpa {

struct AccTcCtx {
  const Trans* rec;     // window-sorted interband records
  const float2* M;      // vertices in sorted order [n_inter][nlf]
  const float2* M2;
  float2* Sdf;          // double-float S0 [nw][np][ncomp] (hi, lo)
  int* status;
  int nlf, nw, obase, wmax, n_inter;
  double domega, eta, cut_over_eta;
  double scaleA;        // power of two folded into w
  float scaleB;         // power of two folded into M2
  float inv_scale;      // 1 / (scaleA scaleB)
  float inv_src;        // 1 / (scale of the pre-split A-side tile)
  int nht;              // G-tiles of the local fields (96 rows, or the chosen tile of the
                        // warp-specialised kernel)
  int sym;              // 1: S0 is Hermitian (complex) or symmetric (real) -- M2 = M --, so only the
                        // tile pairs gi <= gj are computed (blockIdx.y enumerates them) and the
                        // conversion to FP64 mirrors the others
  long long a_chunk, a_tile;  // A-side source: bytes per chunk and per tile
  int a_lo;             // A-side source: offset of the lo rows
  int n_rows;           // rows of M / M2 (n_inter rounded up to a multiple of 32, zero padded)
  int seg;              // chunks accumulated in one TMEM segment before it is read back
  const int* order;     // k_accum_ws: frequency-row blocks in launch order (costliest window
                        // first), null: in index order
};

constexpr int TC_TT = 32;       // transitions per chunk (K = 64 16-bit values)
constexpr int TC_GA = 128;      // G rows per tile (MMA M)
constexpr int TC_GB = 96;       // G' rows per tile
constexpr int TC_FLUSH = 32;    // chunks summed in FP32 before a double-float flush
constexpr uint32_t TC_SPINS = 1u << 16;  // suspending polls: about 1.3 s at most

template <bool F16>
__device__ __forceinline__ void split8(const float* x, uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (F16) {
      __half2 hh = __floats2half2_rn(x[2 * i], x[2 * i + 1]);
      float2 f = __half22float2(hh);
      __half2 ll = __floats2half2_rn(x[2 * i] - f.x, x[2 * i + 1] - f.y);
      h[i] = *reinterpret_cast<uint32_t*>(&hh);
      l[i] = *reinterpret_cast<uint32_t*>(&ll);
    } else {
      __nv_bfloat162 hh = __floats2bfloat162_rn(x[2 * i], x[2 * i + 1]);
      float2 f = __bfloat1622float2(hh);
      __nv_bfloat162 ll = __floats2bfloat162_rn(x[2 * i] - f.x, x[2 * i + 1] - f.y);
      h[i] = *reinterpret_cast<uint32_t*>(&hh);
      l[i] = *reinterpret_cast<uint32_t*>(&ll);
    }
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ void st16(unsigned char* tile, int row, int chunk, uint4 v) {
  *reinterpret_cast<uint4*>(tile + row * 128 + ((chunk ^ (row & 7)) << 4)) = v;
}

__device__ __forceinline__ double lorentz_tc(const AccTcCtx& A, int r, double e1, double e2, bool* in) {
  double o = __dmul_rn((double)(r + A.obase), A.domega);
  double dE = __dadd_rn(__dadd_rn(o, e1), -e2);
  double den = __dadd_rn(__dmul_rn(dE, dE), __dmul_rn(A.eta, A.eta));
  double L = __ddiv_rn(A.eta, den);
  *in = L >= A.cut_over_eta;
  return L;
}

__device__ __forceinline__ int lb_lo(const Trans* rec, int n, int key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (rec[mid].lo < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// (hi, lo) += v in double-float arithmetic (TwoSum then Fast2Sum).
__device__ __forceinline__ float2 df_add(float2 a, float v) {
  float s = __fadd_rn(a.x, v);
  float bb = __fsub_rn(s, a.x);
  float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(v, bb));
  float lo = __fadd_rn(a.y, e);
  float h = __fadd_rn(s, lo);
  float l = __fsub_rn(lo, __fsub_rn(h, s));
  return make_float2(h, l);
}


// Pre-split B tiles of one 32-transition chunk, laid out exactly as the
// 128-byte-swizzled K-major shared-memory tiles the MMA reads, so that a CTA
// fetches them with one bulk copy:
//   tile 0/1: B1 hi/lo, row G' = [ Re b | Im b ]          (b = sB * M2_t(G'))
//   tile 2/3: B2 hi/lo, row G' = [ -Im b | Re b ]         (complex S0 only)
// 96 rows per tile (rows >= nlf are zero), 12 KB per tile.
constexpr uint32_t TC_TILE = TC_GB * 128;


}  // namespace rpa
