// k_accum_ws_r.cu -- the real-S0 (Sloss) instantiations of the
// warp-specialised accumulation kernel, one per tile variant.

#include "k_accum_ws.cuh"

namespace rpa {

int launch_ws_real(rpa_ctx* c, const AccTcCtx& A, int nw, bool sepa, int gb, int nio, const unsigned char* tiles,
                   const unsigned char* tilesA) {
#define RPA_WS_R(GB_, NIO_)                                                                                  \
  if (gb == GB_ && nio == NIO_)                                                                              \
    return sepa ? launch_ws<ws_fit_nio(NIO_, false, true, GB_), false, true, GB_>(c, A, nw, tiles, tilesA)  \
                : launch_ws<NIO_, false, false, GB_>(c, A, nw, tiles, tilesA);
  RPA_WS_R(96, 2)
  RPA_WS_R(128, 1)
  RPA_WS_R(64, 2)
  RPA_WS_R(48, 2)
  RPA_WS_R(32, 2)
#undef RPA_WS_R
  return fail(c, RPA_EINVAL, "accumulation: no real tile variant (%d, %d)", gb, nio);
}

cudaError_t launch_ws_group_real(cudaStream_t s, int device, bool sepa, int gb, int nio, const AccGroupItem* items,
                                 int nitems, long long nctas) {
#define RPA_WSG_R(GB_, NIO_)                                                                                     \
  if (gb == GB_ && nio == NIO_)                                                                                  \
    return sepa ? launch_ws_group<ws_fit_nio(NIO_, false, true, GB_), false, true, GB_>(s, device, items, nitems,  \
                                                                                      nctas)                     \
                : launch_ws_group<NIO_, false, false, GB_>(s, device, items, nitems, nctas);
  RPA_WSG_R(96, 2)
  RPA_WSG_R(128, 1)
  RPA_WSG_R(64, 2)
  RPA_WSG_R(48, 2)
  RPA_WSG_R(32, 2)
#undef RPA_WSG_R
  return cudaErrorInvalidValue;
}

}  // namespace rpa
