// nvtx_ranges.h -- NVTX ranges with the reference's names and ids.
//
// serial_ref annotates its step with NVTX ranges (serial_ref/m_nvtx.f90,
// enabled by EULER2D_NVTX_ANNOTATION_ENABLED): godunov_compute 0
// (m_run.f90:195), compute_dt 1 (:264), convertToPrimitives 2 (:336),
// computeAndStoreFluxes 3 (:387), updateHydro 4 (:502), make_boundaries 5
// (:571).  The C ABI opens the same ranges around the same work, so that a
// timeline of the drop-in lines up with one of the reference.  The ranges
// are host-side (they bracket the launches a call enqueues).
//
// Header-only NVTX3 (shipped with CUDA): with no tool attached a range costs a
// test of a function pointer.  A tool is attached through the environment
// variable NVTX_INJECTION64_PATH (nsys, ncu --nvtx, or any injection
// library).  Build with -DE2D_NVTX=0 to compile the ranges out.
#pragma once

#ifndef E2D_NVTX
#define E2D_NVTX 1
#endif

#if E2D_NVTX
#include <nvtx3/nvToolsExt.h>
#endif

namespace e2d {

enum NvtxId {
  NVTX_GODUNOV = 0,
  NVTX_COMPUTE_DT = 1,
  NVTX_PRIMITIVES = 2,
  NVTX_FLUXES = 3,
  NVTX_UPDATE = 4,
  NVTX_BOUNDARIES = 5,
};

// The range names of serial_ref/m_run.f90, indexed by NvtxId.
inline const char* nvtx_name(int id) {
  static const char* const names[] = {"godunov_compute", "compute_dt", "convertToPrimitives",
                                      "computeAndStoreFluxes", "updateHydro", "make_boundaries"};
  return (id >= 0 && id < 6) ? names[id] : "euler2d";
}

class NvtxRange {
 public:
  explicit NvtxRange(int id) {
#if E2D_NVTX
    // one colour per id, as the reference picks its colour from the id
    static const unsigned colors[] = {0xff00ff00u, 0xff0000ffu, 0xffffff00u, 0xffff00ffu, 0xff00ffffu, 0xffff0000u};
    nvtxEventAttributes_t a = {};
    a.version = NVTX_VERSION;
    a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
    a.colorType = NVTX_COLOR_ARGB;
    a.color = colors[(unsigned)id % 6u];
    a.messageType = NVTX_MESSAGE_TYPE_ASCII;
    a.message.ascii = nvtx_name(id);
    nvtxRangePushEx(&a);
#else
    (void)id;
#endif
  }
  ~NvtxRange() {
#if E2D_NVTX
    nvtxRangePop();
#endif
  }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace e2d
