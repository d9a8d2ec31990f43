// k_accum_ws.cuh -- the warp-specialised tensor-core S0 accumulation.
//
// Same sum as k_accum.cu (Sloss.f90:407-418, Optabs.f90:387-421) as a GEMM
// per frequency row over the transitions whose Lorentzian window holds it.
// One CTA owns NIO consecutive frequency rows and a pair (gi, gj) of G-tiles
// of GB local fields: S_io(G in gi, G' in gj) += A B^T with A = w(t, io) M_t(G)
// (formed per row in shared memory, GB valid rows of the M = 128 MMA) and the
// pre-split B = [B1; B2] (B1 = [Re b | Im b], B2 = [-Im b | Re b], b = M(G'),
// GB rows each; the real S0 of Sloss uses B1 only), one MMA of N = NC GB per
// row and product.  The tile shape (GB, NIO) is a template parameter so that
// small and large NGloc are not forced onto one padding: the host picks it per
// (S0 kind, NGloc, nw) from the autotuner's table or a cost model.
// Roles: one warp streams B tiles and records through an S-stage ring (bulk
// copies, mbarrier transaction counts), one computes the Lorentzian weights,
// one issues the MMAs; twelve warps read back TMEM and form the A tiles.
// Every wait is bounded and ends in an error status.
#pragma once

#include "k_accum_common.cuh"

namespace rpa {

constexpr int WS_SIMT_WARPS = 12;
constexpr int WS_SIMT = 32 * WS_SIMT_WARPS;
constexpr int WS_THREADS = WS_SIMT + 128;
constexpr uint32_t WS_POLLS = 1u << 16;
// register split: 384 x 152 + 128 x 56 = 65536 = 512 x 128 registers at launch (and per SM
// sub-partition 3 x 152 x 32 + 56 x 32 = 16384)
constexpr int WS_REG_SIMT = 152, WS_REG_PROD = 56;

// Bounded wait with a growing sleep between polls, so that waiting warps give
// their issue slots to the warps that form operands.
__device__ __forceinline__ bool ws_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
  uint32_t ns = 32;
  for (uint32_t i = 0; i < WS_POLLS; ++i) {
    if (tc::mbar_try_wait_ns(bar, parity, 20000u)) return true;
    if (*abort_flag) return false;
    __nanosleep(ns);
    ns = ns < 256 ? 2 * ns : 256;
  }
  *abort_flag = 1;
  return false;
}

constexpr uint32_t pow2_at_least(uint32_t x) {
  uint32_t p = 32;
  while (p < x) p *= 2;
  return p;
}

// Whether a shape forms its A tiles in tensor memory: the two TMEM
// accumulator buffers (2 x NIO x NC x GB columns) and two A slots of NIO x
// (hi, lo) x 32 columns (64 K values of 16 bits, two per column) fit the 512
// columns.  Otherwise the A tiles are formed in shared memory.
constexpr bool ws_atmem(int nio, bool cplx, int gb) { return 2 * nio * (cplx ? 2 : 1) * gb + 2 * nio * 64 <= 512; }

// Shared-memory stages of the warp-specialised kernel's ring for a shape
// (the bytes of one stage: pre-split B tiles, separate A-side tiles, records;
// beside them two A slots in shared memory unless they are in TMEM).
constexpr int ws_stages(int nio, bool cplx, bool sepa, int gb) {
  const long long tile = (long long)gb * 128, bsrc = 2LL * (cplx ? 2 : 1) * tile;
  const long long data = (bsrc + (sepa ? 2 * tile : 0) + TC_TT * (long long)sizeof(Trans) + 1023) / 1024 * 1024;
  const long long formed = ws_atmem(nio, cplx, gb) ? 0 : (long long)nio * 2 * TC_GA * 128;
  return (int)((232448 - 2 * formed - 1024 - 3072) / data);
}

// Frequency rows per CTA that fit a shape: nio, or 1 when two stages of the
// ring do not fit beside nio rows of formed A tiles.
constexpr int ws_fit_nio(int nio, bool cplx, bool sepa, int gb) {
  return ws_stages(nio, cplx, sepa, gb) >= 2 ? nio : 1;
}

// Shapes of the warp-specialised kernel for NIO frequency rows per CTA and
// G-tiles of GB local fields (A: GB valid rows of the M = 128 MMA; B: GB rows
// of B1, and of B2 for the complex S0, so one MMA has N = NC * GB).
template <int NIO, bool CPLX, bool SEPA, int GB>
struct WsCfg {
  static constexpr int NC = CPLX ? 2 : 1;
  static constexpr uint32_t A_BYTES = TC_GA * 128;                  // one 16-bit A tile
  static constexpr uint32_t TILE = GB * 128;                        // one 16-bit tile of GB rows
  static constexpr uint32_t BROWS = NC * GB;                        // [B1; B2] or B1
  static constexpr uint32_t BHALF = BROWS * 128;                    // hi (or lo) rows of B
  static constexpr uint32_t BSRC = 2 * BHALF;                       // hi, then lo
  static constexpr uint32_t ASRC = 2 * TILE;                        // separate A-side tiles (M2 != M)
  static constexpr uint32_t REC_OFF = BSRC + (SEPA ? ASRC : 0);
  static constexpr uint32_t DATA = (REC_OFF + TC_TT * sizeof(Trans) + 1023) / 1024 * 1024;
  static constexpr bool ATMEM = ws_atmem(NIO, CPLX, GB);            // A slots in TMEM
  static constexpr uint32_t FORMED = ATMEM ? 0 : NIO * 2 * A_BYTES;  // (Ah, Al) x NIO in shared memory
  static constexpr int S0 = ws_stages(NIO, CPLX, SEPA, GB);
  static constexpr int S = S0 > 6 ? 6 : S0;
  static constexpr size_t SMEM = (size_t)S * DATA + 2 * FORMED + 1024;
  static constexpr uint32_t NMMA = NC * GB;                         // N of one MMA
  static constexpr uint32_t DCOLS = NIO * NMMA;                     // accumulator columns per TMEM buffer
  static constexpr int CW = (int)((DCOLS + 95) / 96 * 32);          // columns per formation thread
  static constexpr uint32_t ACOL = 2 * DCOLS;                       // first TMEM column of the A slots
  static constexpr uint32_t NCOL = pow2_at_least(2 * DCOLS + (ATMEM ? 2 * NIO * 64 : 0));  // TMEM columns allocated
  static_assert(GB % 16 == 0 && GB <= TC_GA, "G tile");
  static_assert(NMMA % 16 == 0 && NMMA <= 256, "MMA N");
  static_assert(DCOLS % 32 == 0 && DCOLS <= 192, "accumulator layout");
};

// The work of one CTA: frequency rows bx * NIO.., tile (pair) by, bz as the
// grid of k_accum_ws numbers them.
template <int NIO, bool CPLX, bool SEPA, int GB>
__device__ __forceinline__ void accum_ws_cta(const AccTcCtx& A, const unsigned char* __restrict__ tiles,
                                             const unsigned char* __restrict__ tilesA, int bx, int by, int bz) {
  using Cfg = WsCfg<NIO, CPLX, SEPA, GB>;
  constexpr int S = Cfg::S;
  constexpr uint32_t DATA = Cfg::DATA, FORMED = Cfg::FORMED, A_BYTES = Cfg::A_BYTES;
  constexpr uint32_t DCOLS = Cfg::DCOLS, NMMA = Cfg::NMMA;  // accumulator columns per TMEM buffer, per MMA
  constexpr int CW = Cfg::CW;                                  // columns per formation thread
  constexpr uint32_t NCOL = Cfg::NCOL;
  static_assert(S >= 2, "shared-memory ring too shallow");
  static_assert(CW % 32 == 0, "accumulator layout");

  extern __shared__ unsigned char smraw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  unsigned char* fbase = base + S * DATA;  // formed slots
  __shared__ uint64_t dfull[S], dfree[S], formed[2], mdone[2], tfree[2], wready[2];
  __shared__ uint32_t tslot;
  __shared__ __align__(16) float wtab[2][NIO][TC_TT];
  __shared__ int range[2];
  __shared__ volatile int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = bx * NIO;
  // G tile (A rows) and G' tile (B rows), 96 local fields each
  int gi = by, gj = bz;
  if (A.sym) {
    // by enumerates the pairs gi <= gj row by row
    int p = by;
    gi = 0;
    while (p >= A.nht - gi) {
      p -= A.nht - gi;
      ++gi;
    }
    gj = gi + p;
  }
  const int nrowA = min(GB, A.nlf - gi * GB);
  const size_t np = (size_t)A.nlf * A.nlf;

  if (warp == 0) {
    tc::tmem_alloc(&tslot, NCOL);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      tc::mbar_init(&dfull[i], 1);
      tc::mbar_init(&dfree[i], WS_SIMT_WARPS + 2);  // formation warps, the weights warp, the MMA commit
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&formed[i], WS_SIMT_WARPS);
      tc::mbar_init(&mdone[i], 1);
      tc::mbar_init(&tfree[i], WS_SIMT_WARPS);
      tc::mbar_init(&wready[i], 1);
    }
    tc::fence_mbar_init();
    abort_flag = 0;
    range[0] = lb_lo(A.rec, A.n_inter, r0 - A.wmax + 1) & ~(TC_TT - 1);
    range[1] = lb_lo(A.rec, A.n_inter, r0 + NIO);
  }
  // A padding rows (G >= nlf) stay zero for the whole kernel (shared-memory A
  // slots; TMEM A slots are written whole for every chunk)
  if constexpr (!Cfg::ATMEM)
    for (uint32_t e = tid; e < 2 * FORMED / 16; e += WS_THREADS)
      reinterpret_cast<uint4*>(fbase)[e] = make_uint4(0, 0, 0, 0);
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t taddr = tslot;
  const int ta = range[0], tb = range[1];
  const int nchunks = (tb - ta + TC_TT - 1) / TC_TT;
  const int chunk0 = ta / TC_TT;
  // Step c of every CTA handles the chunk of its range congruent to c modulo
  // the range length, so CTAs of neighbouring frequency rows (whose ranges
  // overlap almost entirely) read each chunk at the same time and it is
  // fetched from DRAM about once per wave.
  const int rot = nchunks > 0 ? ((-chunk0) % nchunks + nchunks) % nchunks : 0;
  auto phys = [&](int c) { const int p = c + rot; return p >= nchunks ? p - nchunks : p; };

  auto stage = [&](int c) { return base + (size_t)(c % S) * DATA; };
  auto slot = [&](int c) { return fbase + (size_t)(c & 1) * FORMED; };
  bool ok = true;

  if (warp >= WS_SIMT_WARPS) {
    // ---------------- producer / MMA issuer ----------------
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(WS_REG_PROD));
    if (warp == WS_SIMT_WARPS + 2 && lane == 0) {
      // ---------------- loads: a stage is refilled as soon as it is released ----------------
      constexpr uint32_t bytes = Cfg::BSRC + (SEPA ? Cfg::ASRC : 0) + TC_TT * sizeof(Trans);
      int loaded = 0;
      for (; loaded < nchunks && ok; ++loaded) {
        if (loaded >= S) ok = ws_wait(&dfree[loaded % S], ((loaded / S) - 1) & 1, &abort_flag);
        if (!ok) break;
        unsigned char* st = stage(loaded);
        uint64_t* b = &dfull[loaded % S];
        tc::mbar_arrive_expect_tx(b, bytes);
        const int pc = phys(loaded);
        tc::bulk_g2s(st, tiles + ((size_t)(chunk0 + pc) * A.nht + gj) * Cfg::BSRC, Cfg::BSRC, b);
        if (SEPA) {
          const unsigned char* as = tilesA + (size_t)(chunk0 + pc) * A.a_chunk + (size_t)gi * A.a_tile;
          tc::bulk_g2s(st + Cfg::BSRC, as, Cfg::TILE, b);
          tc::bulk_g2s(st + Cfg::BSRC + Cfg::TILE, as + A.a_lo, Cfg::TILE, b);
        }
        tc::bulk_g2s(st + Cfg::REC_OFF, A.rec + ta + (size_t)pc * TC_TT, TC_TT * sizeof(Trans), b);
      }
      if (!ok) {
        abort_flag = 1;
        // bounded wait for the copies in flight before shared memory is released
        for (int c = (loaded > S ? loaded - S : 0); c < loaded; ++c) tc::mbar_wait(&dfull[c % S], (c / S) & 1, 1024);
      }
    }
    if (warp == WS_SIMT_WARPS && lane == 0) {
      // ---------------- MMA issue ----------------
      int issued = 0;
      const uint32_t idesc = tc::idesc_bf16(TC_GA, NMMA, true);
      for (int c = 0; c < nchunks && ok; ++c) {
        ok = ws_wait(&formed[c & 1], (c >> 1) & 1, &abort_flag);
        // an even chunk opens segment c / 2 in TMEM buffer (c / 2) % 2, whose
        // previous segment must have been read back
        if (ok && (c & 1) == 0 && c >= 4) {
          const int sg = (c >> 1) - 2;
          ok = ws_wait(&tfree[sg & 1], (sg >> 1) & 1, &abort_flag);
        }
        if (!ok) break;
        tc::tc_fence_after();
        const uint32_t bh = tc::smem_u32(stage(c)), bl = bh + Cfg::BHALF;
        const uint32_t d0 = taddr + (uint32_t)(((c >> 1) & 1) * DCOLS);
        const uint32_t first = (c & 1) ? 1u : 0u;
        if constexpr (Cfg::ATMEM) {
          // A slot c % 2 in TMEM: per row j, hi in columns 0-31, lo in 32-63
          // (K step ks at column 8 ks)
          const uint32_t a0 = taddr + Cfg::ACOL + (uint32_t)(c & 1) * (uint32_t)(NIO * 64);
#pragma unroll
          for (int j = 0; j < NIO; ++j) {
            const uint32_t ah = a0 + (uint32_t)j * 64u, al = ah + 32u;
            const uint32_t d = d0 + (uint32_t)j * NMMA;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              const uint32_t ko = ks * 32;
              tc::mma_ts(d, ah + ks * 8, tc::desc_sw128(bl + ko), idesc, ks > 0 ? 1u : first);
              tc::mma_ts(d, al + ks * 8, tc::desc_sw128(bh + ko), idesc, 1u);
            }
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) tc::mma_ts(d, ah + ks * 8, tc::desc_sw128(bh + ks * 32), idesc, 1u);
          }
        } else {
        const uint32_t as = tc::smem_u32(slot(c));
#pragma unroll
        for (int j = 0; j < NIO; ++j) {
          const uint32_t ah = as + j * 2 * A_BYTES, al = ah + A_BYTES;
          const uint32_t d = d0 + (uint32_t)j * NMMA;
          // cross products first, the large hi * hi products last
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {
            const uint32_t ko = ks * 32;
            tc::mma_bf16(d, tc::desc_sw128(ah + ko), tc::desc_sw128(bl + ko), idesc, ks > 0 ? 1u : first);
            tc::mma_bf16(d, tc::desc_sw128(al + ko), tc::desc_sw128(bh + ko), idesc, 1u);
          }
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {
            const uint32_t ko = ks * 32;
            tc::mma_bf16(d, tc::desc_sw128(ah + ko), tc::desc_sw128(bh + ko), idesc, 1u);
          }
        }
        }
        tc::mma_commit(&mdone[c & 1]);
        tc::mma_commit(&dfree[c % S]);
        issued = c + 1;
      }
      if (!ok) {
        atomicExch(A.status, 1);
        abort_flag = 1;
        // bounded drain of this CTA's own MMAs
        if (issued > 0) tc::mbar_wait(&mdone[(issued - 1) & 1], ((issued - 1) >> 1) & 1, 1024);
      }
    }
    if (warp == WS_SIMT_WARPS + 1) {
      // ---------------- Lorentzian weights ----------------
      for (int c = 0; c < nchunks && ok; ++c) {
        ok = ws_wait(&dfull[c % S], (c / S) & 1, &abort_flag);
        if (ok && c >= 2) ok = ws_wait(&formed[c & 1], ((c - 2) >> 1) & 1, &abort_flag);  // wtab[c % 2] read
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) break;
        const Trans* rec = reinterpret_cast<const Trans*>(stage(c) + Cfg::REC_OFF);
        const int t = ta + phys(c) * TC_TT + lane;
        const Trans& R = rec[lane];
        const double dE0 = R.e1 - R.e2;
        const float cs = (float)(R.c * A.scaleA) * A.inv_src;
        const float eta = (float)A.eta;
#pragma unroll
        for (int j = 0; j < NIO; ++j) {
          // window membership is the exact [lo, hi] of the record
          const int r = r0 + j;
          float w = 0.f;
          if (t < tb && r < A.nw && r >= R.lo && r <= R.hi) {
            const float dE = (float)fma((double)(r + A.obase), A.domega, dE0);
            w = cs * (eta / fmaf(dE, dE, eta * eta));
          }
          wtab[c & 1][j][lane] = w;
        }
        __syncwarp();
        if (lane == 0) {
          tc::mbar_arrive(&wready[c & 1]);
          tc::mbar_arrive(&dfree[c % S]);
        }
      }
      if (!ok) abort_flag = 1;
    }
  } else {
    // ---------------- read-back, weights, A formation ----------------
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(WS_REG_SIMT));
    // accumulator slice: TMEM lane quadrant wq, columns cg * CW .. cg * CW + CW - 1
    const int wq = warp & 3, cg = warp >> 2;
    const int grow = wq * 32 + lane;       // row of the G tile
    const int gG = gi * GB + grow;         // G
    float acc[CW];
#pragma unroll
    for (int i = 0; i < CW; ++i) acc[i] = 0.f;
    int consumed = 0;
    auto consume = [&](int buf) {
      const uint32_t a0 = taddr + ((uint32_t)(wq * 32) << 16) + (uint32_t)(buf * DCOLS + cg * CW);
#pragma unroll
      for (int p = 0; p < CW / 32; ++p) {
        if (DCOLS % 96 == 0 || cg * CW + 32 * p < (int)DCOLS) {  // the last column group may be short
          float v[32];
          tc::tmem_ld32(a0 + 32 * p, v);
          tc::tmem_ld_wait();
#pragma unroll
          for (int i = 0; i < 32; ++i) acc[32 * p + i] += v[i];
        }
      }
    };
    // column col of the accumulator = (row jr, part, G'): NMMA columns per
    // frequency row, GB per part (Re / Im of the complex S0)
    auto flush = [&]() {
      if (grow < GB && gG < A.nlf) {
        const int ncomp = CPLX ? 2 : 1;
#pragma unroll
        for (int j0 = 0; j0 < CW; j0 += 4) {
          float2* dst[4];
          float2 old[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int col = cg * CW + j0 + j, jr = col / (int)NMMA, cc = col - jr * (int)NMMA;
            const int part = CPLX ? cc / GB : 0, gp = gj * GB + cc - part * GB;
            const int io = r0 + jr, comp = CPLX ? part : 0;
            dst[j] = ((DCOLS % 96 == 0 || col < (int)DCOLS) && gp < A.nlf && io < A.nw)
                         ? A.Sdf + ((size_t)io * np + (size_t)gG + (size_t)A.nlf * gp) * ncomp + comp
                         : nullptr;
            if (dst[j]) old[j] = *dst[j];
          }
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (dst[j]) *dst[j] = df_add(old[j], acc[j0 + j] * A.inv_scale);
        }
      }
#pragma unroll
      for (int j = 0; j < CW; ++j) acc[j] = 0.f;
    };
    for (int c = 0; c < nchunks; ++c) {
      // the weights of chunk c are written after their warp saw the stage
      // land (its arrive releases what it observed), so one wait covers both
      ok = ws_wait(&wready[c & 1], (c >> 1) & 1, &abort_flag);
      if (ok && c >= 2) ok = ws_wait(&mdone[c & 1], ((c - 2) >> 1) & 1, &abort_flag);
      ok = __all_sync(0xffffffffu, ok);
      unsigned char* st = stage(c);
      unsigned char* fs = slot(c);
      if (!ok) break;
      // A tiles: A = w * (hi + lo) of the staged vertex tile (B1 rows, or the
      // separate A-side tile), re-split
      const unsigned char* srch = st + (SEPA ? Cfg::BSRC : 0);
      const unsigned char* srcl = srch + (SEPA ? Cfg::TILE : Cfg::BHALF);
      if constexpr (Cfg::ATMEM) {
        // TMEM A slot c % 2: this thread forms row grow (its lane quadrant) for
        // the 16-bit K chunks ch = cg, cg + 3, cg + 6 (8 K values, 4 columns
        // each); rows >= nrowA are written as zeros
        tc::tc_fence_after();  // the slot's previous MMAs (chunk c - 2) are done
        const uint32_t arow = taddr + ((uint32_t)(wq * 32) << 16) + Cfg::ACOL + (uint32_t)(c & 1) * (uint32_t)(NIO * 64);
        const bool rowok = grow < nrowA;
#pragma unroll
        for (int k3 = 0; k3 < 3; ++k3) {
          const int ch = cg + 3 * k3;
          if (ch < 8) {
            float x[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) x[i] = 0.f;
            if (rowok) {
              const uint32_t off = (uint32_t)grow * 128u + ((uint32_t)(ch ^ (grow & 7)) << 4);
              const uint4 h = *reinterpret_cast<const uint4*>(srch + off);
              const uint4 l = *reinterpret_cast<const uint4*>(srcl + off);
              const uint32_t hw[4] = {h.x, h.y, h.z, h.w}, lw[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                const float2 fh = __half22float2(*reinterpret_cast<const __half2*>(&hw[i]));
                const float2 fl = __half22float2(*reinterpret_cast<const __half2*>(&lw[i]));
                x[2 * i] = fh.x + fl.x;
                x[2 * i + 1] = fh.y + fl.y;
              }
            }
            const int tt0 = (ch & 3) * 8;
#pragma unroll
            for (int j = 0; j < NIO; ++j) {
              const float4 w0 = *reinterpret_cast<const float4*>(&wtab[c & 1][j][tt0]);
              const float4 w1 = *reinterpret_cast<const float4*>(&wtab[c & 1][j][tt0 + 4]);
              const float y[8] = {x[0] * w0.x, x[1] * w0.y, x[2] * w0.z, x[3] * w0.w,
                                  x[4] * w1.x, x[5] * w1.y, x[6] * w1.z, x[7] * w1.w};
              uint4 hi, lo;
              split8<true>(y, hi, lo);
              const uint32_t col = arow + (uint32_t)j * 64u + (uint32_t)ch * 4u;
              tc::tmem_st4(col, hi.x, hi.y, hi.z, hi.w);
              tc::tmem_st4(col + 32u, lo.x, lo.y, lo.z, lo.w);
            }
          }
        }
        tc::tmem_st_wait();
        tc::tc_fence_before();
      } else {
#pragma unroll 2
      for (int e = tid; e < nrowA * 8; e += WS_SIMT) {
        const int row = e >> 3, ch = e & 7;
        const uint32_t off = (uint32_t)row * 128u + ((uint32_t)(ch ^ (row & 7)) << 4);
        const uint4 h = *reinterpret_cast<const uint4*>(srch + off);
        const uint4 l = *reinterpret_cast<const uint4*>(srcl + off);
        float x[8];
        const uint32_t hw[4] = {h.x, h.y, h.z, h.w}, lw[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float2 fh = __half22float2(*reinterpret_cast<const __half2*>(&hw[i]));
          const float2 fl = __half22float2(*reinterpret_cast<const __half2*>(&lw[i]));
          x[2 * i] = fh.x + fl.x;
          x[2 * i + 1] = fh.y + fl.y;
        }
        const int tt0 = (ch & 3) * 8;
#pragma unroll
        for (int j = 0; j < NIO; ++j) {
          const float4 w0 = *reinterpret_cast<const float4*>(&wtab[c & 1][j][tt0]);
          const float4 w1 = *reinterpret_cast<const float4*>(&wtab[c & 1][j][tt0 + 4]);
          const float y[8] = {x[0] * w0.x, x[1] * w0.y, x[2] * w0.z, x[3] * w0.w,
                              x[4] * w1.x, x[5] * w1.y, x[6] * w1.z, x[7] * w1.w};
          uint4 hi, lo;
          split8<true>(y, hi, lo);
          *reinterpret_cast<uint4*>(fs + j * 2 * A_BYTES + off) = hi;
          *reinterpret_cast<uint4*>(fs + j * 2 * A_BYTES + A_BYTES + off) = lo;
        }
      }
      }
      tc::fence_async_smem();
      __syncwarp();
      if (lane == 0) {
        tc::mbar_arrive(&formed[c & 1]);
        tc::mbar_arrive(&dfree[c % S]);
      }
      // chunk c - 2 done: for odd c it closed segment (c - 3) / 2, read back
      // once chunk c is handed over (the MMA warp needs that TMEM buffer only
      // for chunk c + 1)
      if (c >= 3 && (c & 1)) {
        const int sg = (c - 3) >> 1;
        tc::tc_fence_after();
        consume(sg & 1);
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&tfree[sg & 1]);
        if (++consumed % TC_FLUSH == 0) flush();
      }
    }
    // drain: read back the segments the loop did not reach
    if (ok) {
      const int nseg = (nchunks + 1) / 2, ncons = nchunks >= 3 ? (nchunks - 2) / 2 : 0;
      for (int sg = ncons; sg < nseg && ok; ++sg) {
        const int cl = min(2 * sg + 1, nchunks - 1);
        ok = __all_sync(0xffffffffu, ws_wait(&mdone[cl & 1], (cl >> 1) & 1, &abort_flag));
        if (!ok) break;
        tc::tc_fence_after();
        consume(sg & 1);
      }
      if (ok) flush();
    }
    if (!ok) {
      atomicExch(A.status, 1);
      abort_flag = 1;
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}


template <int NIO, bool CPLX, bool SEPA, int GB>
__global__ void __launch_bounds__(WS_THREADS, 1)
    k_accum_ws(AccTcCtx A, const unsigned char* __restrict__ tiles, const unsigned char* __restrict__ tilesA) {
  accum_ws_cta<NIO, CPLX, SEPA, GB>(A, tiles, tilesA, A.order ? A.order[blockIdx.x] : (int)blockIdx.x, blockIdx.y,
                                    blockIdx.z);
}

// Launch order of the frequency-row blocks: costliest window first (chunks
// of records it sweeps, the same range the CTA computes), so that the last
// CTAs to start are short ones.  A row's cost varies ~30-fold along the
// spectrum (few transitions near zero frequency and beyond the band
// widths), and in index order the last wave held full-cost rows.
constexpr int WS_ORDER_MAX = 4096;
static __global__ void __launch_bounds__(1024) k_row_order(const Trans* __restrict__ rec, int n_inter, int wmax, int nrb,
                                                    int nio, int* __restrict__ order) {
  __shared__ unsigned long long key[WS_ORDER_MAX];
  int n = 1;
  while (n < nrb) n <<= 1;
  for (int b = threadIdx.x; b < n; b += blockDim.x) {
    unsigned long long k = ~0ull;  // padding sorts last
    if (b < nrb) {
      const int r0 = b * nio;
      const int ta = lb_lo(rec, n_inter, r0 - wmax + 1) & ~(TC_TT - 1);
      const int tb = lb_lo(rec, n_inter, r0 + nio);
      const unsigned cost = (unsigned)max(0, (tb - ta + TC_TT - 1) / TC_TT);
      k = ((unsigned long long)(~cost) << 32) | (unsigned)b;  // ascending: costliest first, then by index
    }
    key[b] = k;
  }
  __syncthreads();
  // bitonic sort, ascending
  for (int size = 2; size <= n; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const unsigned long long a = key[i], b2 = key[j];
          if ((a > b2) == ((i & size) == 0)) {
            key[i] = b2;
            key[j] = a;
          }
        }
      }
      __syncthreads();
    }
  for (int i = threadIdx.x; i < nrb; i += blockDim.x) order[i] = (int)(key[i] & 0xffffffffu);
}

// Enqueues the row-block order of an accumulation over nrb blocks of nio rows
// into the context's order buffer; *order stays null (index order) when there
// are more blocks than the sort holds.
static int row_order(rpa_ctx* c, const AccTcCtx& A, int nrb, int nio, const int** order) {
  *order = nullptr;
  if (nrb > WS_ORDER_MAX) return RPA_OK;
  RPA_TRY(ensure(c, c->d_order, WS_ORDER_MAX * sizeof(int)));
  k_row_order<<<1, 1024, 0, c->stream>>>(A.rec, A.n_inter, A.wmax, nrb, nio, c->d_order.as<int>());
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  *order = c->d_order.as<int>();
  return RPA_OK;
}

// One item of a grouped launch: the accumulation of one q-point (its launch
// context and pre-split tiles) and the first CTA of the grouped grid that
// works on it; its CTAs are numbered as k_accum_ws's grid (nrb row blocks x
// npy x npz tiles).
struct AccGroupItem {
  AccTcCtx A;
  const unsigned char* tiles;
  const unsigned char* tilesA;
  long long cta0;
  int nrb, npy, npz, pad;
};

// Grouped-tile launch: the S0 accumulations of several q-points (same tile
// shape, each with its own NGloc, nw, transitions and buffers) as one grid.
// A CTA finds its item by binary search over cta0 and copies its context to
// shared memory.
template <int NIO, bool CPLX, bool SEPA, int GB>
__global__ void __launch_bounds__(WS_THREADS, 1)
    k_accum_ws_group(const AccGroupItem* __restrict__ items, int nitems) {
  __shared__ __align__(16) AccGroupItem it;
  __shared__ int sidx;
  if (threadIdx.x == 0) {
    int lo = 0, hi = nitems - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (items[mid].cta0 <= (long long)blockIdx.x) lo = mid;
      else hi = mid - 1;
    }
    sidx = lo;
  }
  __syncthreads();
  {
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(items + sidx);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&it);
    for (int i = threadIdx.x; i < (int)(sizeof(AccGroupItem) / 8); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const long long local = (long long)blockIdx.x - it.cta0;
  const int bl = (int)(local % it.nrb);
  const int bx = it.A.order ? it.A.order[bl] : bl;  // the q-point's row blocks, costliest first
  const long long rest = local / it.nrb;
  accum_ws_cta<NIO, CPLX, SEPA, GB>(it.A, it.tiles, it.tilesA, bx, (int)(rest % it.npy), (int)(rest / it.npy));
}

// Pre-split B operand of the warp-specialised kernel, per chunk and GB-row
// tile of G': the hi rows, then the lo rows; rows 0..GB-1 = [Re b | Im b] (B1),
// rows GB..2GB-1 = [-Im b | Re b] (B2, complex S0 only), b = scale * M(G'),
// rows with G' >= nlf zero.
template <bool CPLX, int GB>
__global__ void k_presplit_ws(const float2* __restrict__ M, int nlf, int nchunks, int nht, float scale,
                              unsigned char* __restrict__ tiles) {
  constexpr uint32_t BROWS = CPLX ? 2 * GB : GB, BHALF = BROWS * 128;
  const long long ntask = (long long)nchunks * nht * GB * 4;
  for (long long task = blockIdx.x * (long long)blockDim.x + threadIdx.x; task < ntask;
       task += (long long)gridDim.x * blockDim.x) {
    const long long cht = task / (GB * 4);
    const int rem = (int)(task % (GB * 4));
    const int ch = (int)(cht / nht), ht = (int)(cht % nht);
    // the four 16-byte groups of a row on neighbouring threads: every warp
    // store fills whole 32-byte sectors of eight rows
    const int row = rem >> 2, grp = rem & 3, g = ht * GB + row;
    float re[8], im[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      float2 m = g < nlf ? M[((size_t)ch * TC_TT + grp * 8 + q) * nlf + g] : make_float2(0.f, 0.f);
      re[q] = m.x * scale;
      im[q] = m.y * scale;
    }
    unsigned char* t = tiles + (size_t)cht * 2 * BHALF;
    uint4 rh, rl, ih, il;
    split8<true>(re, rh, rl);
    split8<true>(im, ih, il);
    st16(t, row, grp, rh);
    st16(t + BHALF, row, grp, rl);
    st16(t, row, 4 + grp, ih);
    st16(t + BHALF, row, 4 + grp, il);
    if (CPLX) {
      const uint32_t sg = 0x80008000u;  // split(-x) = -split(x)
      const int r2 = GB + row;
      st16(t, r2, grp, make_uint4(ih.x ^ sg, ih.y ^ sg, ih.z ^ sg, ih.w ^ sg));
      st16(t + BHALF, r2, grp, make_uint4(il.x ^ sg, il.y ^ sg, il.z ^ sg, il.w ^ sg));
      st16(t, r2, 4 + grp, rh);
      st16(t + BHALF, r2, 4 + grp, rl);
    }
  }
}


template <int NIO, bool CPLX, bool SEPA, int GB>
static int launch_ws(rpa_ctx* c, const AccTcCtx& A, int nw, const unsigned char* tiles, const unsigned char* tilesA) {
  using Cfg = WsCfg<NIO, CPLX, SEPA, GB>;
  auto kern = k_accum_ws<NIO, CPLX, SEPA, GB>;
  RPA_CUDA(c, allow_dynamic_smem(kern, c->device));
  dim3 grid((nw + NIO - 1) / NIO, A.sym ? A.nht * (A.nht + 1) / 2 : A.nht, A.sym ? 1 : A.nht);
  AccTcCtx Ao = A;
  RPA_TRY(row_order(c, A, (int)grid.x, NIO, &Ao.order));
  kern<<<grid, WS_THREADS, Cfg::SMEM, c->stream>>>(Ao, tiles, tilesA);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}


// nctas = 0: only raises the kernel's shared-memory limit (done before a
// stream capture, so the captured launch makes no attribute call).
template <int NIO, bool CPLX, bool SEPA, int GB>
static cudaError_t launch_ws_group(cudaStream_t s, int device, const AccGroupItem* items, int nitems,
                                   long long nctas) {
  using Cfg = WsCfg<NIO, CPLX, SEPA, GB>;
  auto kern = k_accum_ws_group<NIO, CPLX, SEPA, GB>;
  if (nctas == 0) return allow_dynamic_smem(kern, device);
  kern<<<(unsigned)nctas, WS_THREADS, Cfg::SMEM, s>>>(items, nitems);
  return cudaGetLastError();
}

template <bool CPLX, int GB>
static int launch_presplit_ws(rpa_ctx* c, const float2* M, int nchunks, int nht, float scale, unsigned char* tiles) {
  k_presplit_ws<CPLX, GB><<<4096, 256, 0, c->stream>>>(M, c->nlf, nchunks, nht, scale, tiles);
  RPA_CUDA(c, cudaGetLastError());
  ++c->launches;
  return RPA_OK;
}


}  // namespace rpa

namespace rpa {

// Tile variants of the warp-specialised kernel: GB local fields per G-tile,
// NIO frequency rows per CTA.  The first of each list is the default shape.
// (Shapes whose formation warps spill registers are left out.)
struct AccVariant {
  int gb, nio;
};
constexpr AccVariant ACC_VARIANTS_COMPLEX[] = {{96, 1}, {64, 1}, {32, 2}};
constexpr AccVariant ACC_VARIANTS_REAL[] = {{96, 2}, {128, 1}, {64, 2}, {48, 2}, {32, 2}};

// Kernel launch of variant (gb, nio) on pre-split tiles (k_accum_ws_c.cu, k_accum_ws_r.cu).
int launch_ws_complex(rpa_ctx* c, const AccTcCtx& A, int nw, bool sepa, int gb, int nio, const unsigned char* tiles,
                      const unsigned char* tilesA);
int launch_ws_real(rpa_ctx* c, const AccTcCtx& A, int nw, bool sepa, int gb, int nio, const unsigned char* tiles,
                   const unsigned char* tilesA);
// Grouped launch of the real-S0 variant (gb, nio) over nitems items (device
// array) with nctas CTAs in all (k_accum_ws_r.cu); nctas = 0 sets the
// kernel's shared-memory attribute only.
cudaError_t launch_ws_group_real(cudaStream_t s, int device, bool sepa, int gb, int nio, const AccGroupItem* items,
                                 int nitems, long long nctas);
// Pre-split B tiles of GB rows for nchunks chunks and nht tiles.
int presplit_ws_tiles(rpa_ctx* c, bool cplx, int gb, const float2* M, int nchunks, int nht, float scale,
                      unsigned char* tiles);

}  // namespace rpa
