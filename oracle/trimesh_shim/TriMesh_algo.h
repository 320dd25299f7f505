// Stand-in for Trimesh2's TriMesh_algo.h (Trimesh2 2022.03.04 is not installed here).
//
// Test infrastructure only: src/util_io.cpp includes it for one mesh-reading helper
// (src/util_io.cpp:139-141) that oracle/ref_io_shim.cpp never calls; the writers it does call
// (write_binvox, write_vox) use no Trimesh2 code.
#pragma once
#include "TriMesh.h"

namespace trimesh {
inline void reorder_verts(TriMesh*) {}
}  // namespace trimesh
