// k_accum_ws_c.cu -- the complex-S0 (Optabs) instantiations of the
// warp-specialised accumulation kernel, one per tile variant, and the
// pre-split of the B tiles for every G-tile size.

#include "k_accum_ws.cuh"

namespace rpa {

int launch_ws_complex(rpa_ctx* c, const AccTcCtx& A, int nw, bool sepa, int gb, int nio, const unsigned char* tiles,
                      const unsigned char* tilesA) {
#define RPA_WS_C(GB_, NIO_)                                                                                  \
  if (gb == GB_ && nio == NIO_)                                                                              \
    return sepa ? launch_ws<ws_fit_nio(NIO_, true, true, GB_), true, true, GB_>(c, A, nw, tiles, tilesA)    \
                : launch_ws<NIO_, true, false, GB_>(c, A, nw, tiles, tilesA);
  RPA_WS_C(96, 1)
  RPA_WS_C(64, 1)
  RPA_WS_C(32, 2)
#undef RPA_WS_C
  return fail(c, RPA_EINVAL, "accumulation: no complex tile variant (%d, %d)", gb, nio);
}

int presplit_ws_tiles(rpa_ctx* c, bool cplx, int gb, const float2* M, int nchunks, int nht, float scale,
                      unsigned char* tiles) {
  switch (gb) {
    case 128: return cplx ? launch_presplit_ws<true, 128>(c, M, nchunks, nht, scale, tiles)
                          : launch_presplit_ws<false, 128>(c, M, nchunks, nht, scale, tiles);
    case 96: return cplx ? launch_presplit_ws<true, 96>(c, M, nchunks, nht, scale, tiles)
                         : launch_presplit_ws<false, 96>(c, M, nchunks, nht, scale, tiles);
    case 64: return cplx ? launch_presplit_ws<true, 64>(c, M, nchunks, nht, scale, tiles)
                         : launch_presplit_ws<false, 64>(c, M, nchunks, nht, scale, tiles);
    case 48: return cplx ? launch_presplit_ws<true, 48>(c, M, nchunks, nht, scale, tiles)
                         : launch_presplit_ws<false, 48>(c, M, nchunks, nht, scale, tiles);
    case 32: return cplx ? launch_presplit_ws<true, 32>(c, M, nchunks, nht, scale, tiles)
                         : launch_presplit_ws<false, 32>(c, M, nchunks, nht, scale, tiles);
    default: return fail(c, RPA_EINVAL, "accumulation: no pre-split for G-tiles of %d rows", gb);
  }
}

}  // namespace rpa
