// reference_binding.hpp -- what OpenCAMLib itself would call to run its
// drop-cutter on the GB300 library: the C-ABI descriptor of one of its
// cutter objects, a device mesh of one of its STLSurf objects, and the body
// of BatchDropCutter::run() (src/dropcutter/batchdropcutter.cpp:187-231,
// dropCutter5) on the device.  Compiled against OpenCAMLib's own headers
// (reference_binding.cpp; recipe in oracle/Makefile, target `binding`).
#pragma once
#include <vector>

#include "ocl_gb300.h"

namespace ocl {
class MillingCutter;
class STLSurf;
class CLPoint;
}  // namespace ocl

namespace ocl_gb300_binding {

// The constructor arguments of a CylCutter, BallCutter, BullCutter,
// ConeCutter or CompositeCutter (presets included) as the library's cutter
// descriptor.  ConeCutter keeps only length = radius / tan(angle) + l
// (src/cutters/conecutter.cpp:39-49); the l given back is the double for
// which the library's constructor arithmetic returns that length exactly.
// OCL_GB300_UNSUPPORTED_CUTTER for any other MillingCutter subclass.
int cutter_desc(const ocl::MillingCutter& c, ocl_gb300_cutter* out);

// A device mesh of the surface's triangles in STLSurf order.
int mesh_create(const ocl::STLSurf& s, unsigned bucket_size, ocl_gb300_mesh* out);

// BatchDropCutter::run() on the device: every CL point lifted in place, its
// CC point replaced (as CLPoint::liftZ does).
int batch_drop(ocl_gb300_mesh mesh, const ocl::MillingCutter& c, std::vector<ocl::CLPoint>& clpoints,
               ocl_gb300_stats* stats);

}  // namespace ocl_gb300_binding
