// C-ABI shim around the reference's own CPU voxelizer, compiled by oracle/build_ref.sh together
// with the reference's unmodified src/cpu_voxelizer.cpp into oracle/_ref/libref_cpu.so.
//
// Test infrastructure only (the checker, never the product).  It exposes:
//   ref_cpu_voxelize          -> cpu_voxelizer::cpu_voxelize_mesh        (src/cpu_voxelizer.cpp:35)
//   ref_cpu_voxelize_solid    -> cpu_voxelizer::cpu_voxelize_mesh_solid  (src/cpu_voxelizer.cpp:241)
//   ref_create_mesh_bbcube    -> createMeshBBCube                        (src/util.h:80-110)
//   ref_voxinfo_init          -> voxinfo::voxinfo                        (src/util.h:56-61)
//   ref_morton_lut            -> host_morton256_{x,y,z}                  (src/morton_LUTs.h:5,42,78)
// The triangle soup (9 floats per triangle, the layout main.cpp uploads, src/main.cpp:61-80) is
// turned into a fresh Trimesh-like container on every call because the reference shifts the
// vertices in place (src/cpu_voxelizer.cpp:40-45).
#include <cstdint>
#include <cstring>
#include <cstdio>
#include "cpu_voxelizer.h"

static_assert(sizeof(voxinfo) == 64, "voxinfo layout");

static trimesh::TriMesh soup_to_mesh(const float* tris, size_t n) {
	trimesh::TriMesh m;
	m.vertices.resize(3 * n);
	m.faces.resize(n);
	for (size_t i = 0; i < n; i++) {
		for (int k = 0; k < 3; k++) {
			const float* v = tris + 9 * i + 3 * k;
			m.vertices[3 * i + k] = trimesh::point(v[0], v[1], v[2]);
			m.faces[i][k] = static_cast<int>(3 * i + k);
		}
	}
	return m;
}

static voxinfo load_info(const void* info64) {
	alignas(voxinfo) unsigned char buf[sizeof(voxinfo)];
	std::memcpy(buf, info64, sizeof(voxinfo));
	return *reinterpret_cast<voxinfo*>(buf);
}

extern "C" {

void ref_cpu_voxelize(const void* info64, const float* tris, uint32_t* table, int morton) {
	voxinfo info = load_info(info64);
	trimesh::TriMesh m = soup_to_mesh(tris, info.n_triangles);
	cpu_voxelizer::cpu_voxelize_mesh(info, &m, table, morton != 0);
	std::fflush(stdout);
}

void ref_cpu_voxelize_solid(const void* info64, const float* tris, uint32_t* table, int morton) {
	voxinfo info = load_info(info64);
	trimesh::TriMesh m = soup_to_mesh(tris, info.n_triangles);
	cpu_voxelizer::cpu_voxelize_mesh_solid(info, &m, table, morton != 0);
	std::fflush(stdout);
}

void ref_create_mesh_bbcube(const float in_min[3], const float in_max[3], float out_min[3], float out_max[3]) {
	AABox<float3> box(make_float3(in_min[0], in_min[1], in_min[2]), make_float3(in_max[0], in_max[1], in_max[2]));
	AABox<float3> c = createMeshBBCube<float3>(box);
	out_min[0] = c.min.x; out_min[1] = c.min.y; out_min[2] = c.min.z;
	out_max[0] = c.max.x; out_max[1] = c.max.y; out_max[2] = c.max.z;
}

void ref_voxinfo_init(const float bmin[3], const float bmax[3], const uint32_t grid[3], uint64_t n_tri, void* out64) {
	AABox<float3> box(make_float3(bmin[0], bmin[1], bmin[2]), make_float3(bmax[0], bmax[1], bmax[2]));
	voxinfo v(box, make_uint3(grid[0], grid[1], grid[2]), static_cast<size_t>(n_tri));
	std::memset(out64, 0, sizeof(voxinfo));
	std::memcpy(out64, &v, sizeof(voxinfo));
}

void ref_morton_lut(int axis, uint32_t out[256]) {
	const uint32_t* src = axis == 0 ? host_morton256_x : (axis == 1 ? host_morton256_y : host_morton256_z);
	std::memcpy(out, src, 256 * sizeof(uint32_t));
}

}  // extern "C"
