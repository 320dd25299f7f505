// Minimal stand-in for the Trimesh2 container (Trimesh2 2022.03.04 is not installed here).
//
// Test infrastructure only: it lets oracle/build_ref.sh compile the reference's own CPU voxelizer
// (src/cpu_voxelizer.cpp) and its command-line program (src/main.cpp, relinked against libcvx.so)
// unmodified.  The reference touches Trimesh2 only as a container:
// `vertices[i] - move_min` (src/cpu_voxelizer.cpp:44), `faces[i][k]` (:63-65) and the
// x/y/z members read by trimesh_to_float3 (src/util.h:11-14).  No hot-path arithmetic lives in
// Trimesh2; the one float operation it performs here is the per-component subtraction below,
// which is what trimesh::Vec<3,float>::operator- does.
#pragma once
#include <cstdio>
#include <cstdlib>
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
	struct Box {
		point min, max;
	};
	std::vector<point> vertices;
	std::vector<Face> faces;
	Box bbox;

	// What the reference's main() calls (src/main.cpp:166-179): set_verbose, read, need_faces,
	// need_bbox.  read() takes Wavefront OBJ only -- "v x y z" lines and "f" lines of 1-based (or
	// negative, relative) vertex indices with optional /vt/vn parts, polygons split into fans
	// (v0, v[k-1], v[k]) -- enough for the meshes the relinking test writes.
	static void set_verbose(bool) {}
	static TriMesh* read(const char* filename) {
		std::FILE* f = std::fopen(filename, "r");
		if (!f) return nullptr;
		TriMesh* m = new TriMesh();
		char line[8192];
		while (std::fgets(line, sizeof line, f)) {
			if (line[0] == 'v' && (line[1] == ' ' || line[1] == '\t')) {
				float x, y, z;
				if (std::sscanf(line + 2, "%f %f %f", &x, &y, &z) == 3) m->vertices.push_back(point(x, y, z));
			} else if (line[0] == 'f' && (line[1] == ' ' || line[1] == '\t')) {
				std::vector<int> idx;
				char* q = line + 2;
				for (;;) {
					char* end = nullptr;
					const long k = std::strtol(q, &end, 10);
					if (end == q) break;
					idx.push_back(k < 0 ? (int)m->vertices.size() + (int)k : (int)k - 1);
					q = end;
					while (*q && *q != ' ' && *q != '\t' && *q != '\n' && *q != '\r') q++;  // skip /vt/vn
				}
				for (size_t k = 2; k < idx.size(); k++) m->faces.push_back(Face{{idx[0], idx[k - 1], idx[k]}});
			}
		}
		std::fclose(f);
		return m;
	}
	void need_faces() {}
	void need_bbox() {
		if (vertices.empty()) return;
		bbox.min = bbox.max = vertices[0];
		for (const point& v : vertices) {
			bbox.min.x = v.x < bbox.min.x ? v.x : bbox.min.x;
			bbox.min.y = v.y < bbox.min.y ? v.y : bbox.min.y;
			bbox.min.z = v.z < bbox.min.z ? v.z : bbox.min.z;
			bbox.max.x = v.x > bbox.max.x ? v.x : bbox.max.x;
			bbox.max.y = v.y > bbox.max.y ? v.y : bbox.max.y;
			bbox.max.z = v.z > bbox.max.z ? v.z : bbox.max.z;
		}
	}
	bool write(const char*) { return false; }
};

}  // namespace trimesh
