// Minimal stand-in for the Trimesh2 container (Trimesh2 2022.03.04 is not installed here).
//
// Test infrastructure only: it lets oracle/build_ref.sh compile the reference's own CPU voxelizer
// (src/cpu_voxelizer.cpp) unmodified.  The reference touches Trimesh2 only as a container:
// `vertices[i] - move_min` (src/cpu_voxelizer.cpp:44), `faces[i][k]` (:63-65) and the
// x/y/z members read by trimesh_to_float3 (src/util.h:11-14).  No hot-path arithmetic lives in
// Trimesh2; the one float operation it performs here is the per-component subtraction below,
// which is what trimesh::Vec<3,float>::operator- does.
#pragma once
#include <vector>

namespace trimesh {

struct vec3 {
	float x, y, z;
	vec3() : x(0.0f), y(0.0f), z(0.0f) {}
	vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
typedef vec3 point;

struct TriMesh {
	struct Face {
		int v[3];
		int& operator[](int i) { return v[i]; }
		const int& operator[](int i) const { return v[i]; }
	};
	std::vector<point> vertices;
	std::vector<Face> faces;
	// File I/O is not provided (only src/util_io.cpp:140,149 names it, in write_obj_cubes, which
	// the shims never run).
	static TriMesh* read(const char*) { return nullptr; }
	bool write(const char*) { return false; }
};

}  // namespace trimesh
