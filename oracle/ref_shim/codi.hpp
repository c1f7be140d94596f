/* Forward declarations that let the reference's core/codiheader.hh parse
 * without CoDiPack (the operator-overloading AD route is not built). */
#ifndef LBMGPU_REF_CODI_STUB
#define LBMGPU_REF_CODI_STUB
namespace codi {
template <class T> struct LinearIndexHandler;
template <class R, class I> struct ChunkTapeTypes;
template <class T> struct JacobiTape;
template <class T> struct ActiveReal;
}  // namespace codi
#endif
